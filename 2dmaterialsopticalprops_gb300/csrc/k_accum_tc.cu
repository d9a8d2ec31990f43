// k_accum_tc.cu -- spectral accumulation on the tcgen05 tensor cores.
//
// Same sum as k_accum.cu (Sloss.f90:407-418, Optabs.f90:387-421), written per
// frequency row io as a GEMM over the transitions whose Lorentzian window
// contains io (a contiguous range of the window-sorted transitions):
//     S_io(G,G') += sum_t [w(t,io) M_t(G)] conj(M2_t(G'))
// Complex arithmetic is folded into one real GEMM by stacking the K axis
// (32 transitions -> 64 K columns: real parts, then imaginary parts):
//     A(G, :)      = [ Re a_t  | Im a_t ]        a_t = w(t,io) M_t(G)
//     B(G', :)     = [ Re b_t  | Im b_t ]  ->  D(G, G')      = Re S
//     B(96+G', :)  = [ -Im b_t | Re b_t ]  ->  D(G, 96 + G') = Im S
// (the real S0 of Sloss uses the first half only).
//
// Precision.  Operands are split into 16-bit hi + lo halves (fp16 after a
// power-of-two scaling of A and B, or bf16) and D = Ah Bh + Ah Bl + Al Bh.
// The tensor core's FP32 accumulation loses low bits when small products are
// added to a large accumulator, so no accumulator is chained for long: every
// 32-transition chunk starts a fresh TMEM accumulator (two buffers, ping-pong,
// small cross products issued first), the chunk results are summed in FP32
// registers, and every FLUSH chunks those sums are added into a double-float
// (hi + lo FP32) copy of S0 that is converted to FP64 at the end.
//
// Work split.  One CTA owns NIO consecutive frequency rows and a 128 G x 96 G'
// tile.  Per chunk, all 256 threads (i) read the TMEM result of chunk c-2 into
// their register sums, (ii) build the swizzled 16-bit tiles of chunk c while
// the tensor core still runs chunk c-1, and thread 0 then issues chunk c's
// MMAs and commits them to the stage's mbarrier.  Every wait is bounded; on a
// timeout the CTA records an error, waits (bounded) for its own MMAs, frees
// its TMEM and returns.

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstring>

#include "rpa_internal.cuh"
#include "tc05.cuh"

namespace rpa {

struct AccTcCtx {
  const Trans* rec;     // window-sorted interband records
  const float2* M;      // vertices in sorted order [n_inter][nlf]
  const float2* M2;
  float2* Sdf;          // double-float S0 [nw][np][ncomp] (hi, lo)
  int* status;
  int nlf, nw, obase, wmax, n_inter;
  double domega, eta, cut_over_eta;
  double scaleA;        // power of two folded into w
  float scaleB;         // power of two folded into M2
  float inv_scale;      // 1 / (scaleA scaleB)
  float inv_src;        // 1 / (scale of the pre-split A-side tile)
  int nht;              // 96-row tiles of the local fields
  int sym;              // 1: S0 is Hermitian (complex) or symmetric (real) -- M2 = M --, so only the
                        // tile pairs gi <= gj are computed (blockIdx.y enumerates them) and the
                        // conversion to FP64 mirrors the others
  long long a_chunk, a_tile;  // A-side source: bytes per chunk and per tile
  int a_lo;             // A-side source: offset of the lo rows
  int n_rows;           // rows of M / M2 (n_inter rounded up to a multiple of 32, zero padded)
  int seg;              // chunks accumulated in one TMEM segment before it is read back
};

constexpr int TC_TT = 32;       // transitions per chunk (K = 64 16-bit values)
constexpr int TC_GA = 128;      // G rows per tile (MMA M)
constexpr int TC_GB = 96;       // G' rows per tile
constexpr int TC_FLUSH = 32;    // chunks summed in FP32 before a double-float flush
constexpr uint32_t TC_SPINS = 1u << 16;  // suspending polls: about 1.3 s at most

template <bool F16>
__device__ __forceinline__ void split8(const float* x, uint4& hi, uint4& lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (F16) {
      __half2 hh = __floats2half2_rn(x[2 * i], x[2 * i + 1]);
      float2 f = __half22float2(hh);
      __half2 ll = __floats2half2_rn(x[2 * i] - f.x, x[2 * i + 1] - f.y);
      h[i] = *reinterpret_cast<uint32_t*>(&hh);
      l[i] = *reinterpret_cast<uint32_t*>(&ll);
    } else {
      __nv_bfloat162 hh = __floats2bfloat162_rn(x[2 * i], x[2 * i + 1]);
      float2 f = __bfloat1622float2(hh);
      __nv_bfloat162 ll = __floats2bfloat162_rn(x[2 * i] - f.x, x[2 * i + 1] - f.y);
      h[i] = *reinterpret_cast<uint32_t*>(&hh);
      l[i] = *reinterpret_cast<uint32_t*>(&ll);
    }
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

__device__ __forceinline__ void st16(unsigned char* tile, int row, int chunk, uint4 v) {
  *reinterpret_cast<uint4*>(tile + row * 128 + ((chunk ^ (row & 7)) << 4)) = v;
}

__device__ __forceinline__ double lorentz_tc(const AccTcCtx& A, int r, double e1, double e2, bool* in) {
  double o = __dmul_rn((double)(r + A.obase), A.domega);
  double dE = __dadd_rn(__dadd_rn(o, e1), -e2);
  double den = __dadd_rn(__dmul_rn(dE, dE), __dmul_rn(A.eta, A.eta));
  double L = __ddiv_rn(A.eta, den);
  *in = L >= A.cut_over_eta;
  return L;
}

__device__ int lb_lo(const Trans* rec, int n, int key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (rec[mid].lo < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// (hi, lo) += v in double-float arithmetic (TwoSum then Fast2Sum).
__device__ __forceinline__ float2 df_add(float2 a, float v) {
  float s = __fadd_rn(a.x, v);
  float bb = __fsub_rn(s, a.x);
  float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(v, bb));
  float lo = __fadd_rn(a.y, e);
  float h = __fadd_rn(s, lo);
  float l = __fsub_rn(lo, __fsub_rn(h, s));
  return make_float2(h, l);
}

// Pre-split B tiles of one 32-transition chunk, laid out exactly as the
// 128-byte-swizzled K-major shared-memory tiles the MMA reads, so that a CTA
// fetches them with one bulk copy:
//   tile 0/1: B1 hi/lo, row G' = [ Re b | Im b ]          (b = sB * M2_t(G'))
//   tile 2/3: B2 hi/lo, row G' = [ -Im b | Re b ]         (complex S0 only)
// 96 rows per tile (rows >= nlf are zero), 12 KB per tile.
constexpr uint32_t TC_TILE = TC_GB * 128;

template <bool F16, bool CPLX>
__global__ void k_presplit(const float2* __restrict__ M2, int nlf, int nchunks, int nht, float scaleB,
                           unsigned char* __restrict__ tiles) {
  const int ntile = CPLX ? 4 : 2;
  const long long ntask = (long long)nchunks * nht * TC_GB * 4;
  for (long long task = blockIdx.x * (long long)blockDim.x + threadIdx.x; task < ntask;
       task += (long long)gridDim.x * blockDim.x) {
    const int chh = (int)(task / (TC_GB * 4)), rem = (int)(task % (TC_GB * 4));
    const int ch = chh / nht, ht = chh % nht;
    const int row = rem % TC_GB, grp = rem / TC_GB;
    const int g = ht * TC_GB + row;
    float re[8], im[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      float2 m = g < nlf ? M2[((size_t)ch * TC_TT + grp * 8 + q) * nlf + g] : make_float2(0.f, 0.f);
      re[q] = m.x * scaleB;
      im[q] = m.y * scaleB;
    }
    unsigned char* t = tiles + (size_t)chh * ntile * TC_TILE;
    uint4 rh, rl, ih, il;
    split8<F16>(re, rh, rl);
    split8<F16>(im, ih, il);
    st16(t, row, grp, rh);
    st16(t + TC_TILE, row, grp, rl);
    st16(t, row, 4 + grp, ih);
    st16(t + TC_TILE, row, 4 + grp, il);
    if (CPLX) {
      const uint32_t sg = 0x80008000u;  // split(-x) = -split(x)
      st16(t + 2 * TC_TILE, row, grp, make_uint4(ih.x ^ sg, ih.y ^ sg, ih.z ^ sg, ih.w ^ sg));
      st16(t + 3 * TC_TILE, row, grp, make_uint4(il.x ^ sg, il.y ^ sg, il.z ^ sg, il.w ^ sg));
      st16(t + 2 * TC_TILE, row, 4 + grp, rh);
      st16(t + 3 * TC_TILE, row, 4 + grp, rl);
    }
  }
}

// One CTA: NIO frequency rows x (128 G) x (96 G').  Per chunk the bulk copies
// bring the pre-split B tiles, the FP32 vertex rows (for A = w M) and the
// transition records; threads form only the A tiles.
//   complex: D_re = A B1^T (TMEM cols 0..95), D_im = A B2^T (cols 96..191)
//   real:    D(io0) = A(io0) B1^T, D(io1) = A(io1) B1^T
// STAGE_M (nlf <= 96): the FP32 vertex rows come by bulk copy too; otherwise
// the A-forming threads read them from global memory.
template <int NIO, bool CPLX, bool F16, bool STAGE_M>
__global__ void __launch_bounds__(256, 1) k_accum_tc(AccTcCtx A, const unsigned char* __restrict__ tiles) {
  constexpr int NTB = CPLX ? 4 : 2;                          // B tiles per chunk
  constexpr uint32_t A_BYTES = TC_GA * 128;
  constexpr uint32_t BT_BYTES = NTB * TC_TILE;
  constexpr uint32_t STAGE = BT_BYTES + NIO * 2 * A_BYTES;    // B tiles, then (Ah, Al) x NIO
  constexpr int DCOLS = 192;                                 // TMEM columns per buffer
  constexpr uint32_t NCOL = 512;
  static_assert((CPLX ? 2 * NIO : NIO) * TC_GB == DCOLS, "accumulator layout");

  extern __shared__ unsigned char smraw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  float2* mstage = reinterpret_cast<float2*>(base + 2 * STAGE);  // [2][TC_TT][nlf]
  __shared__ __align__(16) Trans rstage[2][TC_TT];
  __shared__ uint64_t bar[2], mbar[2];
  __shared__ uint32_t tslot;
  __shared__ float wtab[2][NIO][TC_TT];
  __shared__ int range[2];

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r0 = blockIdx.x * NIO;
  const int g0 = blockIdx.y * TC_GA, ht = blockIdx.z, h0 = ht * TC_GB, nht = gridDim.z;
  const int nrowA = min(TC_GA, A.nlf - g0), nrowB = min(TC_GB, A.nlf - h0);
  const size_t np = (size_t)A.nlf * A.nlf;

  auto Bt = [&](int s, int i) { return base + s * STAGE + i * TC_TILE; };
  auto Ah = [&](int s, int j) { return base + s * STAGE + BT_BYTES + j * 2 * A_BYTES; };
  auto Al = [&](int s, int j) { return base + s * STAGE + BT_BYTES + j * 2 * A_BYTES + A_BYTES; };

  if (warp == 0) {
    tc::tmem_alloc(&tslot, NCOL);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    tc::fence_mbar_init();
    // chunks start on multiples of 32 rows; the extra leading rows get w = 0
    range[0] = lb_lo(A.rec, A.n_inter, r0 - A.wmax + 1) & ~(TC_TT - 1);
    range[1] = lb_lo(A.rec, A.n_inter, r0 + NIO);
  }
  // A padding rows (G >= nlf) stay zero for the whole kernel
  for (uint32_t e = tid; e < 2 * STAGE / 16; e += 256) reinterpret_cast<uint4*>(base)[e] = make_uint4(0, 0, 0, 0);
  tc::fence_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t taddr = tslot;
  const int ta = range[0], tb = range[1];
  const int nchunks = (tb - ta + TC_TT - 1) / TC_TT;
  const uint32_t idesc = tc::idesc_bf16(TC_GA, TC_GB, F16);
  const uint32_t mbytes = (uint32_t)(TC_TT * A.nlf * sizeof(float2));
  const uint32_t rbytes = (uint32_t)(TC_TT * sizeof(Trans));

  auto prefetch = [&](int c, int buf) {
    const int ts = ta + c * TC_TT;
    tc::mbar_arrive_expect_tx(&mbar[buf], BT_BYTES + (STAGE_M ? mbytes : 0u) + rbytes);
    tc::bulk_g2s(Bt(buf, 0), tiles + ((size_t)(ts / TC_TT) * nht + ht) * BT_BYTES, BT_BYTES, &mbar[buf]);
    if (STAGE_M) tc::bulk_g2s(mstage + (size_t)buf * TC_TT * A.nlf, A.M + (size_t)ts * A.nlf, mbytes, &mbar[buf]);
    tc::bulk_g2s(&rstage[buf][0], A.rec + ts, rbytes, &mbar[buf]);
  };
  if (tid == 0 && nchunks > 0) prefetch(0, 0);

  // this thread's slice of the accumulator: TMEM lane quarter wq, column half hf
  const int wq = warp & 3, hf = warp >> 2;
  const int grow = g0 + wq * 32 + lane;                // G
  const int io_t = CPLX ? r0 : r0 + hf;                // frequency row of this slice
  const int comp = CPLX ? hf : 0;                      // Re / Im
  float acc[96];
#pragma unroll
  for (int i = 0; i < 96; ++i) acc[i] = 0.f;

  auto consume = [&](int buf) {
    float v[96];
    const uint32_t a0 = taddr + ((uint32_t)(wq * 32) << 16) + (uint32_t)(buf * DCOLS + hf * 96);
    tc::tmem_ld32(a0, v);
    tc::tmem_ld32(a0 + 32, v + 32);
    tc::tmem_ld32(a0 + 64, v + 64);
    tc::tmem_ld_wait();
#pragma unroll
    for (int i = 0; i < 96; ++i) acc[i] += v[i];
  };
  auto flush = [&]() {
    if (grow < A.nlf && io_t < A.nw) {
      const int ncomp = CPLX ? 2 : 1;
      float2* rowp = A.Sdf + ((size_t)io_t * np + (size_t)grow + (size_t)A.nlf * h0) * ncomp + comp;
      const size_t step = (size_t)A.nlf * ncomp;
      const int nb = nrowB;
#pragma unroll
      for (int j0 = 0; j0 < 96; j0 += 16) {
        float2 old[16];
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (j0 + j < nb) old[j] = rowp[(j0 + j) * step];
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (j0 + j < nb) rowp[(j0 + j) * step] = df_add(old[j], acc[j0 + j] * A.inv_scale);
      }
    }
#pragma unroll
    for (int j = 0; j < 96; ++j) acc[j] = 0.f;
  };

  bool abort = false;
  int last_commit = -1, consumed = 0;
  const int L = A.seg;

  for (int c = 0; c < nchunks && !abort; ++c) {
    const int s = c & 1;
    const int ts = ta + c * TC_TT;
    if (c >= 2) {
      bool ok = tc::mbar_wait(&bar[s], ((c - 2) >> 1) & 1, TC_SPINS);
      if (!ok) atomicExch(A.status, 1);
      abort = __syncthreads_or(!ok);
      if (abort) break;
      if ((c - 2) % L == L - 1) {  // chunk c-2 closed its segment: read it back
        tc::tc_fence_after();
        consume(((c - 2) / L) & 1);
        tc::tc_fence_before();
        if (++consumed % TC_FLUSH == 0) flush();
      }
    }
    // prefetch chunk c+1 into the stage of chunk c-1 once chunk c-1's MMAs
    // (which read its B tiles) have completed
    if (tid == 0 && c + 1 < nchunks) {
      bool ok = c < 1 || tc::mbar_wait(&bar[s ^ 1], ((c - 1) >> 1) & 1, TC_SPINS);
      if (!ok) atomicExch(A.status, 1);
      else prefetch(c + 1, s ^ 1);
    }
    {
      bool ok = tc::mbar_wait(&mbar[s], (c >> 1) & 1, TC_SPINS);
      if (!ok) atomicExch(A.status, 1);
      abort = __syncthreads_or(!ok);
      if (abort) break;
    }
    // Lorentzian weights of this chunk for the NIO rows (scaled); window
    // membership is the exact [lo, hi] of the record
    if (tid < NIO * TC_TT) {
      int j = tid / TC_TT, tt = tid % TC_TT, t = ts + tt, r = r0 + j;
      float w = 0.f;
      if (t < tb && r < A.nw) {
        const Trans& R = rstage[s][tt];
        if (r >= R.lo && r <= R.hi) {
          float dE = (float)fma((double)(r + A.obase), A.domega, R.e1 - R.e2);
          float eta = (float)A.eta;
          float L2 = eta / fmaf(dE, dE, eta * eta);
          w = (float)(R.c * A.scaleA) * L2;
        }
      }
      wtab[s][j][tt] = w;
    }
    __syncthreads();
    // A tiles: rows G, 8 transitions per task
    const float2* msrc = STAGE_M ? mstage + (size_t)s * TC_TT * A.nlf : A.M + (size_t)ts * A.nlf + g0;
    for (int e = tid; e < nrowA * 4; e += 256) {
      const int row = e % nrowA, grp = e / nrowA;
      float re[8], im[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        float2 m = msrc[(size_t)(grp * 8 + q) * A.nlf + row];
        re[q] = m.x;
        im[q] = m.y;
      }
#pragma unroll
      for (int j = 0; j < NIO; ++j) {
        float xr[8], xi[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          float w = wtab[s][j][grp * 8 + q];
          xr[q] = w * re[q];
          xi[q] = w * im[q];
        }
        uint4 hi, lo;
        split8<F16>(xr, hi, lo);
        st16(Ah(s, j), row, grp, hi);
        st16(Al(s, j), row, grp, lo);
        split8<F16>(xi, hi, lo);
        st16(Ah(s, j), row, 4 + grp, hi);
        st16(Al(s, j), row, 4 + grp, lo);
      }
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::tc_fence_after();
      const uint32_t first = (c % L) == 0 ? 0u : 1u;
      const int dbuf = (c / L) & 1;
#pragma unroll
      for (int j = 0; j < NIO; ++j) {
        const uint32_t ah = tc::smem_u32(Ah(s, j)), al = tc::smem_u32(Al(s, j));
#pragma unroll
        for (int part = 0; part < (CPLX ? 2 : 1); ++part) {
          const uint32_t bh = tc::smem_u32(Bt(s, 2 * part)), bl = tc::smem_u32(Bt(s, 2 * part + 1));
          const uint32_t d = taddr + (uint32_t)(dbuf * DCOLS + (j + part) * TC_GB);
          // cross products first, the large hi*hi products last
#pragma unroll
          for (int ks = 0; ks < 4; ++ks) {
            const uint32_t ko = ks * 32;
            tc::mma_bf16(d, tc::desc_sw128(ah + ko), tc::desc_sw128(bl + ko), idesc, ks > 0 ? 1u : first);
            tc::mma_bf16(d, tc::desc_sw128(al + ko), tc::desc_sw128(bh + ko), idesc, 1u);
          }
#pragma unroll
          for (int ks = 0; ks < 4; ++ks) {
            const uint32_t ko = ks * 32;
            tc::mma_bf16(d, tc::desc_sw128(ah + ko), tc::desc_sw128(bh + ko), idesc, 1u);
          }
        }
      }
      tc::mma_commit(&bar[s]);
    }
    last_commit = c;
  }
  // drain the last (up to) two chunks: read back the segments they close
  if (!abort) {
    for (int cc = (nchunks >= 2 ? nchunks - 2 : 0); cc < nchunks; ++cc) {
      if (!(cc % L == L - 1 || cc == nchunks - 1)) continue;
      const int s = cc & 1;
      bool ok = tc::mbar_wait(&bar[s], (cc >> 1) & 1, TC_SPINS);
      if (!ok) atomicExch(A.status, 1);
      abort = __syncthreads_or(!ok);
      if (abort) break;
      tc::tc_fence_after();
      consume((cc / L) & 1);
      tc::tc_fence_before();
    }
    if (!abort) flush();
  }
  if (abort && tid == 0) {
    // let the MMAs and bulk copies already issued finish before the TMEM and
    // shared memory are released
    if (last_commit >= 0) tc::mbar_wait(&bar[last_commit & 1], (last_commit >> 1) & 1, TC_SPINS);
    for (int b = 0; b < 2; ++b) tc::mbar_wait(&mbar[b], 0, 1024), tc::mbar_wait(&mbar[b], 1, 1024);
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}

// ---------------------------------------------------------------------------
// Warp-specialised form for NGloc <= 96 (one 96-row G' tile holds every local
// field, so the pre-split B tile of a chunk also carries the A-side vertices
// when M2 = M).
//   warpgroup 3, on 56 registers (setmaxnreg) so that the formation warps get
//     152: lane 0 of warp 14 streams the pre-split B tiles and records of each
//     chunk through a ring of S shared-memory stages (bulk copies, mbarrier tx
//     counts), refilling a stage as soon as it is released; lane 0 of warp 12
//     issues chunk c's MMAs as soon as its A tiles are formed and its TMEM
//     buffer has been read back;
//   warp 13: computes the Lorentzian weights of chunk c from its staged
//     records into wtab[c % 2] and hands them over through an mbarrier;
//   warpgroups 0-2 (12 warps): read back the TMEM accumulator of each pair
//     of chunks (a segment) into FP32 register sums (64 of the 192 columns per
//     thread) and form the A tiles of chunk c (w * M, re-split from the staged
//     hi + lo halves) into slot c % 2.
// Precision: a TMEM accumulator sums the 2 x 12 MMAs of one segment (the
// tensor core's FP32 accumulation drops low bits as more products are chained,
// measured 4e-7 for one chunk and 8e-7 for two), the segments are summed in
// FP32 registers and flushed to the double-float S0 every TC_FLUSH segments.
// The complex S0 keeps B1 = [Re b | Im b] and B2 = [-Im b | Re b] as one
// 192-row operand, so D = A [B1; B2]^T is a single N = 192 MMA per product.
// No barrier in the steady state: every hand-off is an mbarrier.  Every wait
// is bounded and gives up early once a timeout has been recorded in the shared
// abort flag.
constexpr int WS_SIMT_WARPS = 12;
constexpr int WS_SIMT = 32 * WS_SIMT_WARPS;
constexpr int WS_THREADS = WS_SIMT + 128;
constexpr uint32_t WS_POLLS = 1u << 16;
// register split: 384 x 152 + 128 x 56 = 65536 = 512 x 128 registers at launch (and per SM
// sub-partition 3 x 152 x 32 + 56 x 32 = 16384)
constexpr int WS_REG_SIMT = 152, WS_REG_PROD = 56;

// Bounded wait with a growing sleep between polls, so that waiting warps give
// their issue slots to the warps that form operands.
__device__ __forceinline__ bool ws_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag) {
  uint32_t ns = 32;
  for (uint32_t i = 0; i < WS_POLLS; ++i) {
    if (tc::mbar_try_wait_ns(bar, parity, 20000u)) return true;
    if (*abort_flag) return false;
    __nanosleep(ns);
    ns = ns < 256 ? 2 * ns : 256;
  }
  *abort_flag = 1;
  return false;
}

template <int NIO, bool CPLX, bool SEPA>
struct WsCfg {
  static constexpr uint32_t A_BYTES = TC_GA * 128;                  // one 16-bit A tile
  static constexpr uint32_t BROWS = CPLX ? 2 * TC_GB : TC_GB;       // [B1; B2] or B1
  static constexpr uint32_t BHALF = BROWS * 128;                    // hi (or lo) rows of B
  static constexpr uint32_t BSRC = 2 * BHALF;                       // hi, then lo
  static constexpr uint32_t ASRC = 2 * TC_TILE;                     // separate A-side tiles (M2 != M)
  static constexpr uint32_t REC_OFF = BSRC + (SEPA ? ASRC : 0);
  static constexpr uint32_t DATA = (REC_OFF + TC_TT * sizeof(Trans) + 1023) / 1024 * 1024;
  static constexpr uint32_t FORMED = NIO * 2 * A_BYTES;             // (Ah, Al) x NIO
  static constexpr int S0 = (int)((232448 - 2 * FORMED - 1024 - 3072) / DATA);
  static constexpr int S = S0 > 6 ? 6 : S0;
  static constexpr size_t SMEM = (size_t)S * DATA + 2 * FORMED + 1024;
};

template <int NIO, bool CPLX, bool SEPA>
__global__ void __launch_bounds__(WS_THREADS, 1)
    k_accum_ws(AccTcCtx A, const unsigned char* __restrict__ tiles, const unsigned char* __restrict__ tilesA) {
  using Cfg = WsCfg<NIO, CPLX, SEPA>;
  constexpr int S = Cfg::S;
  constexpr uint32_t DATA = Cfg::DATA, FORMED = Cfg::FORMED, A_BYTES = Cfg::A_BYTES;
  constexpr uint32_t DCOLS = (CPLX ? 2 : 1) * NIO * TC_GB;  // accumulator columns per TMEM buffer
  constexpr int CW = DCOLS / 3;                                // columns per formation thread
  constexpr uint32_t NCOL = 2 * DCOLS <= 256 ? 256 : 512;
  static_assert(S >= 2, "shared-memory ring too shallow");
  static_assert(CW % 32 == 0, "accumulator layout");

  extern __shared__ unsigned char smraw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  unsigned char* fbase = base + S * DATA;  // formed slots
  __shared__ uint64_t dfull[S], dfree[S], formed[2], mdone[2], tfree[2], wready[2];
  __shared__ uint32_t tslot;
  __shared__ __align__(16) float wtab[2][NIO][TC_TT];
  __shared__ int range[2];
  __shared__ volatile int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r0 = blockIdx.x * NIO;
  // G tile (A rows) and G' tile (B rows), 96 local fields each
  int gi = blockIdx.y, gj = blockIdx.z;
  if (A.sym) {
    // blockIdx.y enumerates the pairs gi <= gj row by row
    int p = blockIdx.y;
    gi = 0;
    while (p >= A.nht - gi) {
      p -= A.nht - gi;
      ++gi;
    }
    gj = gi + p;
  }
  const int nrowA = min(TC_GB, A.nlf - gi * TC_GB);
  const size_t np = (size_t)A.nlf * A.nlf;

  if (warp == 0) {
    tc::tmem_alloc(&tslot, NCOL);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < S; ++i) {
      tc::mbar_init(&dfull[i], 1);
      tc::mbar_init(&dfree[i], WS_SIMT_WARPS + 2);  // formation warps, the weights warp, the MMA commit
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&formed[i], WS_SIMT_WARPS);
      tc::mbar_init(&mdone[i], 1);
      tc::mbar_init(&tfree[i], WS_SIMT_WARPS);
      tc::mbar_init(&wready[i], 1);
    }
    tc::fence_mbar_init();
    abort_flag = 0;
    range[0] = lb_lo(A.rec, A.n_inter, r0 - A.wmax + 1) & ~(TC_TT - 1);
    range[1] = lb_lo(A.rec, A.n_inter, r0 + NIO);
  }
  // A padding rows (G >= nlf) stay zero for the whole kernel
  for (uint32_t e = tid; e < 2 * FORMED / 16; e += WS_THREADS)
    reinterpret_cast<uint4*>(fbase)[e] = make_uint4(0, 0, 0, 0);
  tc::fence_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t taddr = tslot;
  const int ta = range[0], tb = range[1];
  const int nchunks = (tb - ta + TC_TT - 1) / TC_TT;
  const int chunk0 = ta / TC_TT;
  // Step c of every CTA handles the chunk of its range congruent to c modulo
  // the range length, so CTAs of neighbouring frequency rows (whose ranges
  // overlap almost entirely) read each chunk at the same time and it is
  // fetched from DRAM about once per wave.
  const int rot = nchunks > 0 ? ((-chunk0) % nchunks + nchunks) % nchunks : 0;
  auto phys = [&](int c) { const int p = c + rot; return p >= nchunks ? p - nchunks : p; };

  auto stage = [&](int c) { return base + (size_t)(c % S) * DATA; };
  auto slot = [&](int c) { return fbase + (size_t)(c & 1) * FORMED; };
  bool ok = true;

  if (warp >= WS_SIMT_WARPS) {
    // ---------------- producer / MMA issuer ----------------
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(WS_REG_PROD));
    if (warp == WS_SIMT_WARPS + 2 && lane == 0) {
      // ---------------- loads: a stage is refilled as soon as it is released ----------------
      constexpr uint32_t bytes = Cfg::BSRC + (SEPA ? Cfg::ASRC : 0) + TC_TT * sizeof(Trans);
      int loaded = 0;
      for (; loaded < nchunks && ok; ++loaded) {
        if (loaded >= S) ok = ws_wait(&dfree[loaded % S], ((loaded / S) - 1) & 1, &abort_flag);
        if (!ok) break;
        unsigned char* st = stage(loaded);
        uint64_t* b = &dfull[loaded % S];
        tc::mbar_arrive_expect_tx(b, bytes);
        const int pc = phys(loaded);
        tc::bulk_g2s(st, tiles + ((size_t)(chunk0 + pc) * A.nht + gj) * Cfg::BSRC, Cfg::BSRC, b);
        if (SEPA) {
          const unsigned char* as = tilesA + (size_t)(chunk0 + pc) * A.a_chunk + (size_t)gi * A.a_tile;
          tc::bulk_g2s(st + Cfg::BSRC, as, TC_TILE, b);
          tc::bulk_g2s(st + Cfg::BSRC + TC_TILE, as + A.a_lo, TC_TILE, b);
        }
        tc::bulk_g2s(st + Cfg::REC_OFF, A.rec + ta + (size_t)pc * TC_TT, TC_TT * sizeof(Trans), b);
      }
      if (!ok) {
        abort_flag = 1;
        // bounded wait for the copies in flight before shared memory is released
        for (int c = (loaded > S ? loaded - S : 0); c < loaded; ++c) tc::mbar_wait(&dfull[c % S], (c / S) & 1, 1024);
      }
    }
    if (warp == WS_SIMT_WARPS && lane == 0) {
      // ---------------- MMA issue ----------------
      int issued = 0;
      const uint32_t idesc = tc::idesc_bf16(TC_GA, CPLX ? 2 * TC_GB : TC_GB, true);
      for (int c = 0; c < nchunks && ok; ++c) {
        ok = ws_wait(&formed[c & 1], (c >> 1) & 1, &abort_flag);
        // an even chunk opens segment c / 2 in TMEM buffer (c / 2) % 2, whose
        // previous segment must have been read back
        if (ok && (c & 1) == 0 && c >= 4) {
          const int sg = (c >> 1) - 2;
          ok = ws_wait(&tfree[sg & 1], (sg >> 1) & 1, &abort_flag);
        }
        if (!ok) break;
        tc::tc_fence_after();
        const uint32_t bh = tc::smem_u32(stage(c)), bl = bh + Cfg::BHALF;
        const uint32_t as = tc::smem_u32(slot(c));
        const uint32_t d0 = taddr + (uint32_t)(((c >> 1) & 1) * DCOLS);
        const uint32_t first = (c & 1) ? 1u : 0u;
#pragma unroll
        for (int j = 0; j < NIO; ++j) {
          const uint32_t ah = as + j * 2 * A_BYTES, al = ah + A_BYTES;
          const uint32_t d = d0 + (uint32_t)(j * TC_GB);
          // cross products first, the large hi * hi products last
#pragma unroll
          for (int ks = 0; ks < 4; ++ks) {
            const uint32_t ko = ks * 32;
            tc::mma_bf16(d, tc::desc_sw128(ah + ko), tc::desc_sw128(bl + ko), idesc, ks > 0 ? 1u : first);
            tc::mma_bf16(d, tc::desc_sw128(al + ko), tc::desc_sw128(bh + ko), idesc, 1u);
          }
#pragma unroll
          for (int ks = 0; ks < 4; ++ks) {
            const uint32_t ko = ks * 32;
            tc::mma_bf16(d, tc::desc_sw128(ah + ko), tc::desc_sw128(bh + ko), idesc, 1u);
          }
        }
        tc::mma_commit(&mdone[c & 1]);
        tc::mma_commit(&dfree[c % S]);
        issued = c + 1;
      }
      if (!ok) {
        atomicExch(A.status, 1);
        abort_flag = 1;
        // bounded drain of this CTA's own MMAs
        if (issued > 0) tc::mbar_wait(&mdone[(issued - 1) & 1], ((issued - 1) >> 1) & 1, 1024);
      }
    }
    if (warp == WS_SIMT_WARPS + 1) {
      // ---------------- Lorentzian weights ----------------
      for (int c = 0; c < nchunks && ok; ++c) {
        ok = ws_wait(&dfull[c % S], (c / S) & 1, &abort_flag);
        if (ok && c >= 2) ok = ws_wait(&formed[c & 1], ((c - 2) >> 1) & 1, &abort_flag);  // wtab[c % 2] read
        ok = __all_sync(0xffffffffu, ok);
        if (!ok) break;
        const Trans* rec = reinterpret_cast<const Trans*>(stage(c) + Cfg::REC_OFF);
        const int t = ta + phys(c) * TC_TT + lane;
        const Trans& R = rec[lane];
        const double dE0 = R.e1 - R.e2;
        const float cs = (float)(R.c * A.scaleA) * A.inv_src;
        const float eta = (float)A.eta;
#pragma unroll
        for (int j = 0; j < NIO; ++j) {
          // window membership is the exact [lo, hi] of the record
          const int r = r0 + j;
          float w = 0.f;
          if (t < tb && r < A.nw && r >= R.lo && r <= R.hi) {
            const float dE = (float)fma((double)(r + A.obase), A.domega, dE0);
            w = cs * (eta / fmaf(dE, dE, eta * eta));
          }
          wtab[c & 1][j][lane] = w;
        }
        __syncwarp();
        if (lane == 0) {
          tc::mbar_arrive(&wready[c & 1]);
          tc::mbar_arrive(&dfree[c % S]);
        }
      }
      if (!ok) abort_flag = 1;
    }
  } else {
    // ---------------- read-back, weights, A formation ----------------
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(WS_REG_SIMT));
    // accumulator slice: TMEM lane quadrant wq, columns cg * CW .. cg * CW + CW - 1
    const int wq = warp & 3, cg = warp >> 2;
    const int grow = wq * 32 + lane;       // row of the G tile
    const int gG = gi * TC_GB + grow;      // G
    float acc[CW];
#pragma unroll
    for (int i = 0; i < CW; ++i) acc[i] = 0.f;
    int consumed = 0;
    auto consume = [&](int buf) {
      const uint32_t a0 = taddr + ((uint32_t)(wq * 32) << 16) + (uint32_t)(buf * DCOLS + cg * CW);
#pragma unroll
      for (int p = 0; p < CW / 32; ++p) {
        float v[32];
        tc::tmem_ld32(a0 + 32 * p, v);
        tc::tmem_ld_wait();
#pragma unroll
        for (int i = 0; i < 32; ++i) acc[32 * p + i] += v[i];
      }
    };
    // column col of the accumulator = (part, G'): part = Re / Im (complex) or
    // the frequency row of the pair (real)
    auto flush = [&]() {
      if (grow < TC_GB && gG < A.nlf) {
        const int ncomp = CPLX ? 2 : 1;
#pragma unroll
        for (int j0 = 0; j0 < CW; j0 += 4) {
          float2* dst[4];
          float2 old[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int col = cg * CW + j0 + j, part = col / TC_GB, gp = gj * TC_GB + col - part * TC_GB;
            const int io = CPLX ? r0 : r0 + part, comp = CPLX ? part : 0;
            dst[j] = (gp < A.nlf && io < A.nw)
                         ? A.Sdf + ((size_t)io * np + (size_t)gG + (size_t)A.nlf * gp) * ncomp + comp
                         : nullptr;
            if (dst[j]) old[j] = *dst[j];
          }
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (dst[j]) *dst[j] = df_add(old[j], acc[j0 + j] * A.inv_scale);
        }
      }
#pragma unroll
      for (int j = 0; j < CW; ++j) acc[j] = 0.f;
    };
    for (int c = 0; c < nchunks; ++c) {
      ok = ws_wait(&dfull[c % S], (c / S) & 1, &abort_flag);
      if (ok && c >= 2) ok = ws_wait(&mdone[c & 1], ((c - 2) >> 1) & 1, &abort_flag);
      ok = __all_sync(0xffffffffu, ok);
      unsigned char* st = stage(c);
      unsigned char* fs = slot(c);
      // chunk c-2 done: its slot is free, and for odd c it closed segment
      // (c - 3) / 2, which is read back now
      if (ok && c >= 3 && (c & 1)) {
        const int sg = (c - 3) >> 1;
        tc::tc_fence_after();
        consume(sg & 1);
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&tfree[sg & 1]);
        if (++consumed % TC_FLUSH == 0) flush();
      }
      if (ok) ok = __all_sync(0xffffffffu, ws_wait(&wready[c & 1], (c >> 1) & 1, &abort_flag));
      if (!ok) break;
      // A tiles: A = w * (hi + lo) of the staged vertex tile (B1 rows, or the
      // separate A-side tile), re-split
      const unsigned char* srch = st + (SEPA ? Cfg::BSRC : 0);
      const unsigned char* srcl = srch + (SEPA ? TC_TILE : Cfg::BHALF);
#pragma unroll 2
      for (int e = tid; e < nrowA * 8; e += WS_SIMT) {
        const int row = e >> 3, ch = e & 7;
        const uint32_t off = (uint32_t)row * 128u + ((uint32_t)(ch ^ (row & 7)) << 4);
        const uint4 h = *reinterpret_cast<const uint4*>(srch + off);
        const uint4 l = *reinterpret_cast<const uint4*>(srcl + off);
        float x[8];
        const uint32_t hw[4] = {h.x, h.y, h.z, h.w}, lw[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float2 fh = __half22float2(*reinterpret_cast<const __half2*>(&hw[i]));
          const float2 fl = __half22float2(*reinterpret_cast<const __half2*>(&lw[i]));
          x[2 * i] = fh.x + fl.x;
          x[2 * i + 1] = fh.y + fl.y;
        }
        const int tt0 = (ch & 3) * 8;
#pragma unroll
        for (int j = 0; j < NIO; ++j) {
          const float4 w0 = *reinterpret_cast<const float4*>(&wtab[c & 1][j][tt0]);
          const float4 w1 = *reinterpret_cast<const float4*>(&wtab[c & 1][j][tt0 + 4]);
          const float y[8] = {x[0] * w0.x, x[1] * w0.y, x[2] * w0.z, x[3] * w0.w,
                              x[4] * w1.x, x[5] * w1.y, x[6] * w1.z, x[7] * w1.w};
          uint4 hi, lo;
          split8<true>(y, hi, lo);
          *reinterpret_cast<uint4*>(fs + j * 2 * A_BYTES + off) = hi;
          *reinterpret_cast<uint4*>(fs + j * 2 * A_BYTES + A_BYTES + off) = lo;
        }
      }
      tc::fence_async_smem();
      __syncwarp();
      if (lane == 0) {
        tc::mbar_arrive(&formed[c & 1]);
        tc::mbar_arrive(&dfree[c % S]);
      }
    }
    // drain: read back the segments the loop did not reach
    if (ok) {
      const int nseg = (nchunks + 1) / 2, ncons = nchunks >= 3 ? (nchunks - 2) / 2 : 0;
      for (int sg = ncons; sg < nseg && ok; ++sg) {
        const int cl = min(2 * sg + 1, nchunks - 1);
        ok = __all_sync(0xffffffffu, ws_wait(&mdone[cl & 1], (cl >> 1) & 1, &abort_flag));
        if (!ok) break;
        tc::tc_fence_after();
        consume(sg & 1);
      }
      if (ok) flush();
    }
    if (!ok) {
      atomicExch(A.status, 1);
      abort_flag = 1;
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}

// Pre-split B operand of the warp-specialised kernel, per chunk and 96-row
// tile of G': the hi rows, then the lo rows; rows 0-95 = [Re b | Im b] (B1),
// rows 96-191 = [-Im b | Re b] (B2, complex S0 only), b = scale * M(G'),
// rows with G' >= nlf zero.
template <bool CPLX>
__global__ void k_presplit_ws(const float2* __restrict__ M, int nlf, int nchunks, int nht, float scale,
                              unsigned char* __restrict__ tiles) {
  constexpr uint32_t BROWS = CPLX ? 2 * TC_GB : TC_GB, BHALF = BROWS * 128;
  const long long ntask = (long long)nchunks * nht * TC_GB * 4;
  for (long long task = blockIdx.x * (long long)blockDim.x + threadIdx.x; task < ntask;
       task += (long long)gridDim.x * blockDim.x) {
    const long long cht = task / (TC_GB * 4);
    const int rem = (int)(task % (TC_GB * 4));
    const int ch = (int)(cht / nht), ht = (int)(cht % nht);
    // the four 16-byte groups of a row on neighbouring threads: every warp
    // store fills whole 32-byte sectors of eight rows
    const int row = rem >> 2, grp = rem & 3, g = ht * TC_GB + row;
    float re[8], im[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      float2 m = g < nlf ? M[((size_t)ch * TC_TT + grp * 8 + q) * nlf + g] : make_float2(0.f, 0.f);
      re[q] = m.x * scale;
      im[q] = m.y * scale;
    }
    unsigned char* t = tiles + (size_t)cht * 2 * BHALF;
    uint4 rh, rl, ih, il;
    split8<true>(re, rh, rl);
    split8<true>(im, ih, il);
    st16(t, row, grp, rh);
    st16(t + BHALF, row, grp, rl);
    st16(t, row, 4 + grp, ih);
    st16(t + BHALF, row, 4 + grp, il);
    if (CPLX) {
      const uint32_t sg = 0x80008000u;  // split(-x) = -split(x)
      const int r2 = TC_GB + row;
      st16(t, r2, grp, make_uint4(ih.x ^ sg, ih.y ^ sg, ih.z ^ sg, ih.w ^ sg));
      st16(t + BHALF, r2, grp, make_uint4(il.x ^ sg, il.y ^ sg, il.z ^ sg, il.w ^ sg));
      st16(t, r2, 4 + grp, rh);
      st16(t + BHALF, r2, 4 + grp, rl);
    }
  }
}

__global__ void k_cmax(const Trans* __restrict__ rec, int n, unsigned long long* cmax) {
  double mx = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) mx = fmax(mx, fabs(rec[i].c));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(cmax, (unsigned long long)__double_as_longlong(mx));
}

__global__ void k_df_to_f64(const float2* __restrict__ Sdf, double* __restrict__ S, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    float2 v = Sdf[e];
    S[e] += (double)v.x + (double)v.y;
  }
}

// The same conversion for an S0 whose tile pairs gi > gj were not computed
// (M2 = M): entry (G, G') of such a pair is taken from (G', G), conjugated for
// the complex S0 (S(G', G) = sum w M(G') conj M(G) = conj S(G, G')).
template <bool CPLX>
__global__ void k_df_to_f64_sym(const float2* __restrict__ Sdf, double* __restrict__ S, int nw, int nlf,
                                int tile) {
  const size_t np = (size_t)nlf * nlf, n = (size_t)nw * np;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const size_t io = e / np;
    const int p = (int)(e - io * np), iG = p % nlf, jG = p / nlf;
    const bool mirror = iG / tile > jG / tile;
    const size_t src = mirror ? io * np + (size_t)jG + (size_t)nlf * iG : e;
    if (CPLX) {
      const float2 re = Sdf[2 * src], im = Sdf[2 * src + 1];
      const double vi = (double)im.x + (double)im.y;
      S[2 * e] += (double)re.x + (double)re.y;
      S[2 * e + 1] += mirror ? -vi : vi;
    } else {
      const float2 v = Sdf[src];
      S[e] += (double)v.x + (double)v.y;
    }
  }
}

template <int NIO, bool CPLX, bool F16, bool STAGE_M>
static int launch_tc(rpa_ctx* c, const AccTcCtx& A, int nw, const unsigned char* tiles) {
  constexpr int NTB = CPLX ? 4 : 2;
  constexpr size_t STAGE = (size_t)NTB * TC_TILE + (size_t)NIO * 2 * TC_GA * 128;
  const size_t smem = 2 * STAGE + 1024 + (STAGE_M ? 2 * (size_t)TC_TT * A.nlf * sizeof(float2) : 0);
  auto kern = k_accum_tc<NIO, CPLX, F16, STAGE_M>;
  RPA_CUDA(c, allow_dynamic_smem(kern, c->device));
  dim3 grid((nw + NIO - 1) / NIO, (A.nlf + TC_GA - 1) / TC_GA, (A.nlf + TC_GB - 1) / TC_GB);
  kern<<<grid, 256, smem, c->stream>>>(A, tiles);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

template <int NIO, bool CPLX, bool SEPA>
static int launch_ws(rpa_ctx* c, const AccTcCtx& A, int nw, const unsigned char* tiles, const unsigned char* tilesA) {
  using Cfg = WsCfg<NIO, CPLX, SEPA>;
  auto kern = k_accum_ws<NIO, CPLX, SEPA>;
  RPA_CUDA(c, allow_dynamic_smem(kern, c->device));
  dim3 grid((nw + NIO - 1) / NIO, A.sym ? A.nht * (A.nht + 1) / 2 : A.nht, A.sym ? 1 : A.nht);
  kern<<<grid, WS_THREADS, Cfg::SMEM, c->stream>>>(A, tiles, tilesA);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

template <bool CPLX>
static int launch_presplit_ws(rpa_ctx* c, const float2* M, int nchunks, int nht, float scale, unsigned char* tiles) {
  k_presplit_ws<CPLX><<<4096, 256, 0, c->stream>>>(M, c->nlf, nchunks, nht, scale, tiles);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

template <bool F16, bool CPLX>
static int launch_presplit(rpa_ctx* c, const float2* M2, int nchunks, float scaleB, unsigned char* tiles) {
  const int nht = (c->nlf + TC_GB - 1) / TC_GB;
  k_presplit<F16, CPLX><<<4096, 256, 0, c->stream>>>(M2, c->nlf, nchunks, nht, scaleB, tiles);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

static double pow2_floor(double x) { return std::ldexp(1.0, (int)std::floor(std::log2(x))); }

// Interband accumulation of one k-chunk into the double-float S0 (d_Sdf).
int accumulate_tc(rpa_ctx* c, const Chi0Plan& P, int n_inter, int wmax, const float2* Mf, const float2* Mf2,
                  float amaxM, float amaxM2, double cmax) {
  if (n_inter == 0) return RPA_OK;
  AccTcCtx A;
  A.sym = 0;
  A.rec = c->d_sorted.as<Trans>();
  A.M = Mf;
  A.M2 = Mf2;
  A.Sdf = c->d_Sdf.as<float2>();
  A.status = c->d_flags.as<int>() + 2;
  A.nlf = c->nlf;
  A.nw = P.nw;
  A.obase = P.wbase;
  A.wmax = wmax;
  A.n_inter = n_inter;
  A.domega = P.domega;
  A.eta = P.eta;
  A.cut_over_eta = P.cut / P.eta;
  const bool f16 = c->split_f16;
  // |A| <= cmax/eta * |M| * sqrt2, |B| <= |M2| * sqrt2: aim both maxima at ~2^14
  double amA = cmax / P.eta * (double)amaxM * 1.5, amB = (double)amaxM2 * 1.5;
  A.scaleA = (f16 && amA > 0) ? 16384.0 / pow2_floor(amA) : 1.0;
  A.scaleB = (f16 && amB > 0) ? (float)(16384.0 / pow2_floor(amB)) : 1.0f;
  A.inv_scale = (float)(1.0 / (A.scaleA * (double)A.scaleB));
  A.n_rows = (n_inter + TC_TT - 1) / TC_TT * TC_TT;
  A.seg = c->tc_seg > 0 ? c->tc_seg : 1;
  const bool cplx = P.mode == RPA_MODE_CURRENT;
  const int nch = A.n_rows / TC_TT + 1;  // one spare chunk for the last prefetch
  const int nht = (c->nlf + TC_GB - 1) / TC_GB;
  const bool two = Mf2 != Mf;
  if (f16 && A.seg == 1) {
    // warp-specialised kernel on 96-row tiles of G and G'.  The A side reads
    // the B1 rows of the same stage when there is one tile and M2 = M, else
    // its own pre-split source tile (the B tiles of tile gi, or a pre-split
    // copy of M for the yz / zy pair).
    const size_t bsrc = (size_t)(cplx ? 4 : 2) * TC_TILE;
    RPA_TRY(ensure(c, c->d_tiles, (size_t)nch * nht * bsrc));
    unsigned char* tiles = c->d_tiles.as<unsigned char>();
    RPA_TRY(cplx ? launch_presplit_ws<true>(c, Mf2, nch, nht, A.scaleB, tiles)
                 : launch_presplit_ws<false>(c, Mf2, nch, nht, A.scaleB, tiles));
    const unsigned char* tilesA = tiles;
    A.nht = nht;
    A.inv_src = 1.0f / A.scaleB;
    A.a_chunk = (long long)nht * bsrc;
    A.a_tile = (long long)bsrc;
    A.a_lo = (cplx ? 2 : 1) * TC_TILE;
    if (two) {
      const double amS = (double)amaxM * 1.5;
      const float sM = amS > 0 ? (float)(16384.0 / pow2_floor(amS)) : 1.0f;
      RPA_TRY(ensure(c, c->d_tilesA, (size_t)nch * nht * 2 * TC_TILE));
      RPA_TRY(launch_presplit<true, false>(c, Mf, nch, sM, c->d_tilesA.as<unsigned char>()));
      tilesA = c->d_tilesA.as<unsigned char>();
      A.inv_src = 1.0f / sM;
      A.a_chunk = (long long)nht * 2 * TC_TILE;
      A.a_tile = 2 * TC_TILE;
      A.a_lo = TC_TILE;
    }
    const bool sepa = two || nht > 1;
    A.sym = (!two && nht > 1) ? 1 : 0;
    c->s_sym = A.sym != 0;
    if (cplx) return sepa ? launch_ws<1, true, true>(c, A, P.nw, tiles, tilesA) : launch_ws<1, true, false>(c, A, P.nw, tiles, tilesA);
    return sepa ? launch_ws<1, false, true>(c, A, P.nw, tiles, tilesA) : launch_ws<2, false, false>(c, A, P.nw, tiles, tilesA);
  }
  const size_t tbytes = (size_t)nch * nht * (cplx ? 4 : 2) * TC_TILE;
  RPA_TRY(ensure(c, c->d_tiles, tbytes));
  unsigned char* tiles = c->d_tiles.as<unsigned char>();
  const bool st = c->nlf <= TC_GB;  // whole vertex rows fit the bulk-copy staging
  if (cplx) {
    RPA_TRY(f16 ? launch_presplit<true, true>(c, Mf2, nch, A.scaleB, tiles)
                : launch_presplit<false, true>(c, Mf2, nch, A.scaleB, tiles));
    if (st) return f16 ? launch_tc<1, true, true, true>(c, A, P.nw, tiles) : launch_tc<1, true, false, true>(c, A, P.nw, tiles);
    return f16 ? launch_tc<1, true, true, false>(c, A, P.nw, tiles) : launch_tc<1, true, false, false>(c, A, P.nw, tiles);
  }
  RPA_TRY(f16 ? launch_presplit<true, false>(c, Mf2, nch, A.scaleB, tiles)
              : launch_presplit<false, false>(c, Mf2, nch, A.scaleB, tiles));
  if (st) return f16 ? launch_tc<2, false, true, true>(c, A, P.nw, tiles) : launch_tc<2, false, false, true>(c, A, P.nw, tiles);
  return f16 ? launch_tc<2, false, true, false>(c, A, P.nw, tiles) : launch_tc<2, false, false, false>(c, A, P.nw, tiles);
}

__global__ void k_inverse_perm(const int* __restrict__ order, int* __restrict__ pos_of, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) pos_of[order[i]] = i;
}

// Qeff += c M conj(M2) over the intraband rows [t_begin, t_end) of the sorted
// FP32 vertices (one (G,G') element per thread, rows in emission order).
__global__ void k_qeff_f32(const Trans* __restrict__ rec, int t_begin, int t_end, const float2* __restrict__ M,
                           const float2* __restrict__ M2, int nlf, double2* __restrict__ Q) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nlf * nlf) return;
  int gi = p % nlf, gj = p / nlf;
  double qr = 0.0, qi = 0.0;
  for (int t = t_begin; t < t_end; ++t) {
    float2 a = M[(size_t)t * nlf + gi], b = M2[(size_t)t * nlf + gj];
    double xr = (double)a.x * b.x + (double)a.y * b.y, xi = (double)a.y * b.x - (double)a.x * b.y;
    double cc = rec[t].c;
    qr += cc * xr;
    qi += cc * xi;
  }
  double2 v = Q[p];
  v.x += qr;
  v.y += qi;
  Q[p] = v;
}

int inverse_perm(rpa_ctx* c, int n, int* pos_of) {
  if (n == 0) return RPA_OK;
  k_inverse_perm<<<(n + 255) / 256, 256, 0, c->stream>>>(c->d_vals_alt.as<int>(), pos_of, n);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

int qeff_f32(rpa_ctx* c, int n_inter, int n_trans, const float2* Mf, const float2* Mf2) {
  if (n_trans <= n_inter) return RPA_OK;
  int np = c->nlf * c->nlf;
  k_qeff_f32<<<(np + 127) / 128, 128, 0, c->stream>>>(c->d_sorted.as<Trans>(), n_inter, n_trans, Mf, Mf2, c->nlf,
                                                      c->d_Q.as<double2>());
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

// max |c| over the interband records (for the power-of-two operand scaling)
int cmax_of(rpa_ctx* c, int n_inter, double* cmax) {
  *cmax = 0.0;
  if (n_inter == 0) return RPA_OK;
  unsigned long long* d = reinterpret_cast<unsigned long long*>(c->d_ntrans.as<char>() + 8);
  RPA_CUDA(c, cudaMemsetAsync(d, 0, 8, c->stream));
  k_cmax<<<256, 256, 0, c->stream>>>(c->d_sorted.as<Trans>(), n_inter, d);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  RPA_CUDA(c, cudaMemcpyAsync(cmax, d, 8, cudaMemcpyDeviceToHost, c->stream));
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  return RPA_OK;
}

int df_to_f64(rpa_ctx* c, size_t n, int nw, bool cplx) {
  if (c->s_sym) {
    if (cplx)
      k_df_to_f64_sym<true><<<2048, 256, 0, c->stream>>>(c->d_Sdf.as<float2>(), c->d_S.as<double>(), nw, c->nlf,
                                                         TC_GB);
    else
      k_df_to_f64_sym<false><<<2048, 256, 0, c->stream>>>(c->d_Sdf.as<float2>(), c->d_S.as<double>(), nw, c->nlf,
                                                          TC_GB);
  } else {
    k_df_to_f64<<<2048, 256, 0, c->stream>>>(c->d_Sdf.as<float2>(), c->d_S.as<double>(), n);
  }
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

}  // namespace rpa
