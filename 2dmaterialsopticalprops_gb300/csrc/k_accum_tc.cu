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

#include <algorithm>

#include "k_accum_ws.cuh"

namespace rpa {

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

template <bool F16, bool CPLX>
static int launch_presplit(rpa_ctx* c, const float2* M2, int nchunks, float scaleB, unsigned char* tiles) {
  const int nht = (c->nlf + TC_GB - 1) / TC_GB;
  k_presplit<F16, CPLX><<<4096, 256, 0, c->stream>>>(M2, c->nlf, nchunks, nht, scaleB, tiles);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}


static double pow2_floor(double x) { return std::ldexp(1.0, (int)std::floor(std::log2(x))); }

// Cost model of a tile variant, in issue cycles per chunk summed over the
// CTAs of one launch: per CTA and 32-transition chunk the MMAs take ~6 cycles
// per accumulator column (three split products, four K steps of N = NC GB per
// row) and the formation ~8 cycles per valid A row per row, overlapped, plus
// ~200 cycles of hand-off; a launch has ceil(nw / NIO) x (tile pairs) CTAs.
static double acc_model_cost(bool cplx, int nlf, int nw, AccVariant v) {
  const int nht = (nlf + v.gb - 1) / v.gb;
  v.nio = ws_fit_nio(v.nio, cplx, nht > 1, v.gb);
  const double pairs = nht > 1 ? 0.5 * nht * (nht + 1) : 1.0;
  const double rows_avg = (double)nlf / nht;
  const double mma = 6.0 * v.nio * (cplx ? 2 : 1) * v.gb, form = 8.0 * v.nio * std::min<double>(v.gb, rows_avg);
  return std::ceil((double)nw / v.nio) * pairs * (std::max(mma, form) + 200.0);
}

// Tile variant of an accumulation: forced for the context (opts.reserved[2] or
// the autotuner's trial), the autotuner's table entry for (S0 kind, NGloc,
// nw / 64), else the cheapest variant of the cost model.  The yz / zy pair
// (M2 != M) keeps the default 96-row tiles.
static AccVariant acc_variant(rpa_ctx* c, int nw, bool cplx, bool two) {
  if (two) return {TC_GB, 1};
  if (c->acc_force.gb > 0) return {c->acc_force.gb, c->acc_force.nio};
  const auto it = c->acc_table.find(acc_tune_key(cplx, c->nlf, nw));
  if (it != c->acc_table.end()) return {it->second.gb, it->second.nio};
  const AccVariant* list = cplx ? ACC_VARIANTS_COMPLEX : ACC_VARIANTS_REAL;
  const int n = cplx ? (int)(sizeof ACC_VARIANTS_COMPLEX / sizeof(AccVariant))
                     : (int)(sizeof ACC_VARIANTS_REAL / sizeof(AccVariant));
  AccVariant best = list[0];
  double bc = acc_model_cost(cplx, c->nlf, nw, best);
  for (int i = 1; i < n; ++i) {
    const double k = acc_model_cost(cplx, c->nlf, nw, list[i]);
    if (k < 0.9 * bc) {  // the default unless a variant is clearly cheaper
      bc = k;
      best = list[i];
    }
  }
  return best;
}

int acc_variant_list(bool cplx, int* gb, int* nio, int cap) {
  const AccVariant* list = cplx ? ACC_VARIANTS_COMPLEX : ACC_VARIANTS_REAL;
  const int n = cplx ? (int)(sizeof ACC_VARIANTS_COMPLEX / sizeof(AccVariant))
                     : (int)(sizeof ACC_VARIANTS_REAL / sizeof(AccVariant));
  for (int i = 0; i < n && i < cap; ++i) {
    gb[i] = list[i].gb;
    nio[i] = list[i].nio;
  }
  return n;
}

// Interband accumulation of one k-chunk into the double-float S0 (d_Sdf).
int accumulate_tc(rpa_ctx* c, const Chi0Plan& P, int n_inter, int wmax, const float2* Mf, const float2* Mf2,
                  float amaxM, float amaxM2, double cmax) {
  if (n_inter == 0) return RPA_OK;
  AccTcCtx A;
  A.sym = 0;
  A.order = nullptr;
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
    // warp-specialised kernel on G-tiles of v.gb rows.  The A side reads the
    // B1 rows of the same stage when there is one tile and M2 = M, else its
    // own pre-split source tile (the B tiles of tile gi, or a pre-split copy
    // of M for the yz / zy pair, which keeps the 96-row default tile).
    const AccVariant v = acc_variant(c, P.nw, cplx, two);
    const int gb = v.gb, nhv = (c->nlf + gb - 1) / gb;
    const size_t tile = (size_t)gb * 128, bsrc = (size_t)(cplx ? 4 : 2) * tile;
    RPA_TRY(ensure(c, c->d_tiles, (size_t)nch * nhv * bsrc));
    unsigned char* tiles = c->d_tiles.as<unsigned char>();
    RPA_TRY(presplit_ws_tiles(c, cplx, gb, Mf2, nch, nhv, A.scaleB, tiles));
    const unsigned char* tilesA = tiles;
    A.nht = nhv;
    A.inv_src = 1.0f / A.scaleB;
    A.a_chunk = (long long)nhv * bsrc;
    A.a_tile = (long long)bsrc;
    A.a_lo = (cplx ? 2 : 1) * (int)tile;
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
    const bool sepa = two || nhv > 1;
    A.sym = (!two && nhv > 1) ? 1 : 0;
    c->s_sym = A.sym != 0;
    c->s_gb = gb;
    c->acc_last_gb = gb;
    c->acc_last_nio = ws_fit_nio(v.nio, cplx, sepa, gb);
    if (c->defer_acc) {
      // batch mode: describe the launch instead of making it
      AccGroupItem it;
      std::memset(&it, 0, sizeof it);
      it.A = A;
      it.tiles = tiles;
      it.tilesA = tilesA;
      it.nrb = (P.nw + c->acc_last_nio - 1) / c->acc_last_nio;
      it.npy = A.sym ? nhv * (nhv + 1) / 2 : nhv;
      it.npz = A.sym ? 1 : nhv;
      // its row blocks costliest first, computed now on this context's stream
      // (its own order buffer; the batch synchronises the stream before the
      // grouped launch)
      RPA_TRY(row_order(c, A, it.nrb, c->acc_last_nio, &it.A.order));
      static_assert(sizeof(AccGroupItem) <= sizeof(c->deferred_item), "deferred item storage");
      std::memcpy(c->deferred_item, &it, sizeof it);
      c->deferred = true;
      c->deferred_gb = gb;
      c->deferred_nio = v.nio;
      c->deferred_nw = P.nw;
      c->deferred_sepa = sepa;
      c->deferred_cplx = cplx;
      return RPA_OK;
    }
    return cplx ? launch_ws_complex(c, A, P.nw, sepa, gb, v.nio, tiles, tilesA)
                : launch_ws_real(c, A, P.nw, sepa, gb, v.nio, tiles, tilesA);
  }
  if (c->defer_acc) return fail(c, RPA_EINVAL, "accumulation: a deferred (batched) accumulation needs the default fp16 split and TMEM segments");
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
                                                         c->s_gb);
    else
      k_df_to_f64_sym<false><<<2048, 256, 0, c->stream>>>(c->d_Sdf.as<float2>(), c->d_S.as<double>(), nw, c->nlf,
                                                          c->s_gb);
  } else {
    k_df_to_f64<<<2048, 256, 0, c->stream>>>(c->d_Sdf.as<float2>(), c->d_S.as<double>(), n);
  }
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

}  // namespace rpa
