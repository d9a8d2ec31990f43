// k_vertex_mn.cu -- plane-wave vertices on the tcgen05 tensor cores with both
// operands MN-major (mixed path, default vertex kernel).
//
// Same vertices as k_vertex.cu (genMnmK1K2, Sloss.f90:883-952; genStrujniVrhovi,
// Optabs.f90:1354-1472), per FBZ k-point as a GEMM over plane waves:
//     D((G,a), b) = sum_i x_a(G,i) conj(y_b(i))
// x: the gathered side, coefficients of bands a at basis positions map(G,i);
// y: the sequential side, coefficients of bands b at plane wave i.
//   Optabs, and Sloss with more occupied than empty bands: x = C2[m] of K2 at
//     Gfast(G,i), y = C1[n] of K1, i over the plane waves of K1  -> M = D.
//   Sloss with fewer occupied bands (the usual case): x = C1[n] of K1 at the
//     inverse map (the K1 plane wave that Gfast sends to plane wave p of K2),
//     y = C2[m] of K2, p over the plane waves of K2 -> M = conj(D).  The inverse
//     exists because Gfast(G, .) is injective (G'' is an affine bijection of the
//     K1 plane wave); gathering the occupied side moves nocc instead of
//     nbnd - nocc bands per gathered plane wave.
// The coefficients live as four fp16 planes per plane wave, [re_hi, im_hi,
// re_lo, im_lo][bands] (x 2^14), so a gathered plane wave is one contiguous run
// of bands.  The MMA operands are MN-major: a K row of the X tile holds 128
// (G, band) rows, 8 bands per 16-byte chunk, so each gathered (G, plane wave,
// plane) lands with 16-byte cp.async copies and no transposition.  K order in a
// chunk of 32 plane waves: rows 0-31 real parts, 32-63 imaginary parts, so
//     Re D = X[Re] . Re y + X[Im] . Im y,   Im D = X[Im] . Re y - X[Re] . Im y
// Current vertices: the factor separates, f(G,i) = a(G) + b(i), and the column
// blocks of y are [c | b1 c | b2 c] (b c precomputed per launch, split like the
// coefficient planes; b2 c only when two Cartesian components are wanted --
// the yz / zy pair, or a second polarisation prefetched beside the first,
// which then shares the gathers of X and the D[c] block); a(G) multiplies the
// c block at read-back: M_mu = a_mu(G) D[c] + D[b_mu c].
// One or two column blocks (charge; current, one component): the Y tile holds
// [y | y'] with y' = (-Im y rows 0-31, Re y rows 32-63), written by the threads
// that copy the y chunk, and three MMAs of N = 2 NYN per K step give
// Re D = X . y and Im D = X . y'.  Three blocks (k_vertex_mn_split): [y | y']
// would not leave room for enough stages, so the Y tile holds y alone; per K
// step (16 rows) three MMAs of N = NYN give Re D from the same K rows of X and
// Y, and three more give Im D from X's rows and the other half of Y's K rows, negated
// (instruction-descriptor bit) where X holds real parts.
// Small products first: Xl . Yh, Xh . Yl, Xh . Yh.  (The tensor core reads its
// operands from shared memory at 128 bytes per cycle: an N = 128 MMA just
// keeps up.)  Each local-field tile sweeps the plane waves in the opposite
// direction of the previous one, so the coefficient rows read last are read
// again first while they are still in L2.
// Each chunk goes into a fresh TMEM accumulator that the worker warps add to
// FP32 registers; a ring of accumulators (four, two when 192 columns wide)
// keeps the MMA warp from waiting for the read-back of the chunk before last.
// Warp roles: 16 worker warps gather chunk t + S - 1 into the ring of S
// shared-memory stages and read back chunk t - 1 from TMEM; warp 16 issues
// the MMAs.  Every wait is bounded and ends in an error status.

#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>

#include "rpa_internal.cuh"
#include "tc05.cuh"

namespace rpa {

int build_gmap(rpa_ctx* c, int k0, int nk, int nsum_max, int16_t* gmap, int nsum_legacy);
int build_ginv(rpa_ctx* c, int k0, int nk, int nsum_max, int16_t* ginv);

struct VtxMnCtx {
  const int* kmap;
  const double* ktot;
  const double* Glf;
  const int* npw;
  const __half* planes;   // [kibz][npwx][4][nbp]
  const __half* ybt;      // [k_local][nsum_max][4][nbp]: b(i) c split like the planes (current vertices)
  const __half* ybt2;     // the same for the second Cartesian component (three column blocks)
  const int16_t* map;     // [k_local][nlf][nsum_max]: gathered-side position of (G, i), -1 none
  const Trans* trans;
  const long long* offsets;
  const int* pos_of;
  float2* M;
  float2* M2;             // vertex rows of the second component (three column blocks)
  int* ptab_g;            // [k_local][32][NBY]: pair table of the three-block pass (global memory)
  unsigned* amax;         // [2]: max |M|, max |M2| (float bits)
  int* status;
  int k0, nlf, npwx, nbp, nsum_max, legacy, nsum_legacy;
  int swap;               // 1: x = bands n of K1 (inverse map), y = bands m of K2
  int xs, xb, xo0, xo1;   // gathered window: first band, rows per G (multiple of 8), owned bands
  int ys, yo0, yo1;       // sequential window: first band (multiple of 8), owned bands
  int gpt;                // local fields per 128-row tile
  int comp, comp2;         // Cartesian components of b(i) c and b2(i) c
  double q0, q1, q2, Gcar;
  float a_scale, out_scale;
};

constexpr int VM_WORKERS = 512;                 // 16 worker warps
constexpr int VM_THREADS = VM_WORKERS + 32;     // + the MMA warp
constexpr int VM_I = 32;                        // plane waves per chunk (K = 64)
constexpr uint32_t VM_SPINS = 1u << 16;         // suspending polls: about 1.3 s at most
constexpr int VM_SMEM_MAX = 232448 - 1024;      // dynamic shared memory left beside the static part
constexpr int VM_SMAX = 6;

// NB column blocks of y: 1 = charge (y), 2 = current (c, b c), 3 = current
// with a second component (c, b1 c, b2 c).
template <int NBY, int NB>
struct VmCfg {
  static constexpr bool IMG = NB <= 2;                   // y' images in the Y tile
  // three blocks: the Y tile in the 64-byte swizzle (32-wide atoms, no padding
  // to 64 columns) and the pair table in global memory, so that four stages fit
  static constexpr bool SW64 = !IMG;
  static constexpr int NYN = NB * NBY;                   // columns of Re D (and of Im D)
  static constexpr int NYT = IMG ? 2 * NYN : NYN;        // columns of the Y tile
  static constexpr int AW = SW64 ? 32 : 64;              // atom width along N (elements)
  static constexpr uint32_t AB = SW64 ? 512 : 1024;      // bytes of one atom (8 K rows)
  static constexpr int NTA = (NYT + AW - 1) / AW;        // atoms along N of one half (lo or hi) of Y
  static constexpr uint32_t XH = 64 * 128 * 2;           // one half (hi or lo) of X
  static constexpr uint32_t YKG = 2u * NTA * AB;         // Y bytes per group of 8 K rows: hi atoms, then lo atoms
  static constexpr uint32_t YLO = (uint32_t)NTA * AB;    // offset of the lo atoms in a K group
  static constexpr uint32_t STAGE = 2 * XH + 8 * YKG;
  static constexpr bool PTAB_SMEM = IMG;
  static constexpr uint32_t PTAB = PTAB_SMEM ? 32 * NBY * 4 : 0;  // int32 [32][NBY]
  static constexpr int S0 = (int)((VM_SMEM_MAX - 1024 - (int)PTAB) / (int)STAGE);
  static constexpr int S = S0 > VM_SMAX ? VM_SMAX : S0;
  // accumulator columns: Re D then Im D (with images: one MMA of N = 64 NTA over both)
  static constexpr uint32_t N2 = IMG ? 64 * NTA : 2 * NYN;
  static constexpr int NBUF = N2 <= 128 ? 4 : 2;         // TMEM accumulators in the ring
  static constexpr uint32_t NCOL = NBUF * N2 <= 256 ? 256 : 512;
  static constexpr int CW = NBY / 4;                     // columns per thread per block
  static constexpr size_t SMEM = (size_t)S * STAGE + PTAB + 1024;
  static_assert(NBY % 16 == 0 && (SW64 || NTA <= 2) && NYN <= 256, "window too wide");
  static_assert(NBUF * N2 <= 512, "accumulator ring beyond TMEM");
  static_assert(S >= 3, "shared-memory ring too shallow");
  // four stages or more: a step signals the chunk issued S - 2 steps before
  // it waits for the read-back of the chunk before last (see the worker loop)
  static constexpr bool EARLY = S >= 4;
  static_assert(IMG || EARLY, "three blocks need four stages");
  static_assert(PTAB_SMEM || NBY <= 32, "the global pair table holds 32 x 32 entries per k-point");
};

__device__ __forceinline__ void cp16z(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp4(uint32_t dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ uint4 lds16(uint32_t a) {
  uint4 v;
  asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(a));
  return v;
}
__device__ __forceinline__ void sts16(uint32_t a, uint4 v) {
  asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
               : "memory");
}
__device__ __forceinline__ float lds_f32(uint32_t a) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory");
}

// CW consecutive TMEM columns of this thread's lane
template <int CW>
__device__ __forceinline__ void tmem_ld_n(uint32_t addr, float* v) {
  if constexpr (CW >= 16) {
    tc::tmem_ld16(addr, v);
    if constexpr (CW > 16) tmem_ld_n<CW - 16>(addr + 16, v + 16);
  } else if constexpr (CW >= 8) {
    tc::tmem_ld8(addr, v);
    if constexpr (CW > 8) tmem_ld_n<CW - 8>(addr + 8, v + 8);
  } else {
    static_assert(CW == 4, "columns per thread");
    tc::tmem_ld4(addr, v);
  }
}

// the vertex rows of CW consecutive columns of band row a of the pair table
template <int CW>
__device__ __forceinline__ void load_rows(const int* ptab, int (&rr)[CW]) {
  static_assert(CW % 4 == 0, "pair-table row slice");
  const int4* pt = reinterpret_cast<const int4*>(ptab);
#pragma unroll
  for (int q = 0; q < CW / 4; ++q) {
    const int4 w = pt[q];
    rr[4 * q] = w.x;
    rr[4 * q + 1] = w.y;
    rr[4 * q + 2] = w.z;
    rr[4 * q + 3] = w.w;
  }
}

// One CTA per FBZ k-point of the launch.
template <int NBY, int NB>
__global__ void __launch_bounds__(VM_THREADS, 1) k_vertex_mn(VtxMnCtx V) {
  using Cfg = VmCfg<NBY, NB>;
  constexpr bool CURRENT = NB > 1;
  static_assert(Cfg::IMG && Cfg::PTAB_SMEM, "three column blocks run in k_vertex_mn_split");
  constexpr int NP = CURRENT ? NB - 1 : 1;  // vertex sets written
  constexpr int S = Cfg::S, NYN = Cfg::NYN, CW = Cfg::CW;
  constexpr uint32_t XH = Cfg::XH, YKG = Cfg::YKG, YLO = Cfg::YLO, STAGE = Cfg::STAGE;

  extern __shared__ unsigned char smraw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  const uint32_t sbase = tc::smem_u32(base);
  int* ptab = reinterpret_cast<int*>(base + (size_t)S * STAGE);  // [a][b]: vertex row of the pair, -1 none
  __shared__ uint64_t full[VM_SMAX], done[Cfg::NBUF], tfree[Cfg::NBUF];
  __shared__ uint32_t tslot;
  __shared__ volatile int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int kl = blockIdx.x, ik = V.k0 + kl;
  const long long t0 = V.offsets[kl], t1 = V.offsets[kl + 1];
  if (t1 == t0) return;
  const int* km = V.kmap + 5 * ik;
  const int K1 = km[0], K2 = km[2];
  const int kX = V.swap ? K1 : K2, kY = V.swap ? K2 : K1;
  const int nsum = V.legacy ? V.nsum_legacy : V.npw[kY];
  const int nchunk = (nsum + VM_I - 1) / VM_I;
  const int GPT = V.gpt, XB = V.xb;
  const int ngt = (V.nlf + GPT - 1) / GPT;
  const int total = ngt * nchunk;

  if (warp == 0) {
    tc::tmem_alloc(&tslot, Cfg::NCOL);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int s = 0; s < S; ++s) tc::mbar_init(&full[s], VM_WORKERS / 32);
    for (int b = 0; b < Cfg::NBUF; ++b) {
      tc::mbar_init(&done[b], 1);
      tc::mbar_init(&tfree[b], VM_WORKERS / 32);
    }
    abort_flag = 0;
    tc::fence_mbar_init();
  }
  for (int e = tid; e < XB * NBY; e += VM_THREADS) ptab[e] = -1;
  __syncthreads();
  for (long long t = t0 + tid; t < t1; t += VM_THREADS) {
    const int nm = V.trans[t].nm;
    const int n = nm & 0xffff, m = nm >> 16;
    const int xa = V.swap ? n : m, yb = V.swap ? m : n;
    if (xa >= V.xo0 && xa < V.xo1 && yb >= V.yo0 && yb < V.yo1)
      ptab[(xa - V.xs) * NBY + (yb - V.ys)] = V.pos_of[t];
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t taddr = tslot;

  if (warp == VM_WORKERS / 32) {
    // ---------------------------------------------------------------- MMA warp
    if (lane == 0) {
      constexpr uint32_t N2 = Cfg::N2;
      constexpr int NBF = Cfg::NBUF;
      constexpr uint64_t YG2 = 2 * (YKG >> 4);  // descriptor step of 16 K rows of Y
      // one MMA of N = 64 NTA over [y | y']
      const uint32_t id = tc::idesc_f16_mn(128, N2, false);
      // descriptors of stage 0; a chunk adds its byte offsets / 16 to the start-address field
      const uint64_t dx0 = tc::desc_sw128_mn(sbase, 1024u, 2048u);
      const uint64_t dy0 = tc::desc_sw128_mn(sbase + 2 * XH, 1024u, YKG);
      // the next chunk's barriers are tested while this chunk's MMAs are
      // queued (a test costs ~150-200 cycles under the kernel's shared-memory
      // load); only one not yet seen complete is waited for between chunks
      int last = -1;
      int s = 0, ph = 0;
      bool fnext = false, tnext = false;
      for (int t = 0; t < total; ++t) {
        if ((t & 15) == 0 && abort_flag) break;
        if ((!fnext && !tc::mbar_wait(&full[s], (uint32_t)ph, VM_SPINS)) ||
            (!tnext && t >= NBF && !tc::mbar_wait(&tfree[t % NBF], (uint32_t)((t / NBF - 1) & 1), VM_SPINS))) {
          atomicExch(V.status, 1);
          abort_flag = 1;
          break;
        }
        tc::tc_fence_after();
        const int sn = s + 1 == S ? 0 : s + 1;
        const int phn = sn == 0 ? ph ^ 1 : ph;
        const uint64_t so = (uint64_t)(((uint32_t)s * STAGE) >> 4);
        const uint64_t dx = dx0 + so, dy = dy0 + so;
        const uint32_t d = taddr + (uint32_t)((t % NBF) * N2);
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          const uint64_t xh = dx + (uint64_t)(ks * 256), xl = xh + (XH >> 4);
          const uint64_t yh = dy + (uint64_t)ks * YG2, yl = yh + (YLO >> 4);
          const uint32_t acc = ks > 0 ? 1u : 0u;
          tc::mma_bf16(d, xl, yh, id, acc);  // Xl . Yh
          tc::mma_bf16(d, xh, yl, id, 1u);   // + Xh . Yl
          tc::mma_bf16(d, xh, yh, id, 1u);   // + Xh . Yh
          if (ks == 1) fnext = t + 1 >= total || tc::mbar_test_wait(&full[sn], (uint32_t)phn);
          if (ks == 2)
            tnext = t + 1 < NBF || tc::mbar_test_wait(&tfree[(t + 1) % NBF], (uint32_t)(((t + 1) / NBF - 1) & 1));
        }
        tc::mma_commit(&done[t % NBF]);
        last = t;
        s = sn;
        ph = phn;
      }
      if (last >= 0) tc::mbar_wait(&done[last % NBF], (uint32_t)((last / NBF) & 1), VM_SPINS);
    }
  } else {
    // ------------------------------------------------------------- worker warps
    // X copies of this thread: plane wave xpw of the chunk, rows 8 xj .. 8 xj + 7,
    // the four planes (u = 0..3 -> half u / 2, K rows (u % 2) 32 + xpw)
    const int xpw = tid >> 4, xj = tid & 15;
    const int xrow = 8 * xj, xg = xrow / XB, xb0 = xrow - xg * XB;
    const bool xok = xg < GPT && V.xs + xb0 < V.nbp;
    const uint32_t xoff = (uint32_t)(xpw >> 3) * 2048u + (uint32_t)(xj >> 3) * 1024u + (uint32_t)(xpw & 7) * 128u +
                          ((uint32_t)((xj & 7) ^ (xpw & 7)) << 4);
    const size_t pstride = (size_t)4 * V.nbp;  // halves per plane wave
    const __half* xsrc = V.planes + (size_t)kX * V.npwx * pstride + V.xs + xb0;
    const int16_t* mp = V.map + (size_t)kl * V.nlf * V.nsum_max + xpw;
    // Y copies: e = tid + VM_WORKERS v over 2 halves x 64 K rows x NYN / 8 chunks
    constexpr int YCH = NYN / 8, YE = 128 * YCH, YV = (YE + VM_WORKERS - 1) / VM_WORKERS;
    const __half* ysrc_c = V.planes + (size_t)kY * V.npwx * pstride;
    const __half* ysrc_b1 = CURRENT ? V.ybt + (size_t)kl * V.nsum_max * pstride : nullptr;
    // per copy: its place in y (and y'), its source for chunk 0 (a chunk adds
    // its plane-wave offset), the chunk start from which it is a zero fill
    // (beyond nsum, or a band beyond the window), the imaginary-part flag
    uint32_t ydst[YV], yidst[YV];  // the chunk in y, its image in y'
    const __half* ysb[YV];
    int ylim[YV];
    bool ycp[YV], yneg[YV];
#pragma unroll
    for (int v = 0; v < YV; ++v) {
      const int e = tid + VM_WORKERS * v;
      ycp[v] = yneg[v] = false;
      ysb[v] = ysrc_c;
      ylim[v] = 0;
      ydst[v] = yidst[v] = 0;
      if (e < YE) {
        const int line = e / YCH, j = e - line * YCH;
        const int half = line >> 6, kk = line & 63, part = kk >> 5, pw = kk & 31;
        const int col = 8 * j, u = 2 * half + part;
        const int blk = col / NBY;
        const int band = V.ys + col - blk * NBY;
        ydst[v] = 2 * XH + (uint32_t)(kk >> 3) * YKG + (uint32_t)half * YLO + (uint32_t)(col >> 6) * 1024u +
                  (uint32_t)(kk & 7) * 128u + ((uint32_t)(((col >> 3) & 7) ^ (kk & 7)) << 4);
        const int ki = kk ^ 32, ci = NYN + col;  // y' row and column of the chunk
        yidst[v] = 2 * XH + (uint32_t)(ki >> 3) * YKG + (uint32_t)half * YLO + (uint32_t)(ci >> 6) * 1024u +
                   (uint32_t)(ki & 7) * 128u + ((uint32_t)(((ci >> 3) & 7) ^ (ki & 7)) << 4);
        const __half* bp = blk == 0 ? ysrc_c : ysrc_b1;
        ycp[v] = true;
        yneg[v] = part != 0;
        ysb[v] = bp + (size_t)pw * pstride + (band < V.nbp ? u * V.nbp + band : 0);
        ylim[v] = band < V.nbp ? nsum - pw : 0;
      }
    }

    // y' images of the chunks this thread copied into a stage
    constexpr uint32_t NEG = 0x80008000u;
    auto form = [&](int stage) {
      const uint32_t st = sbase + (uint32_t)stage * STAGE;
#pragma unroll
      for (int v = 0; v < YV; ++v) {
        if (!ycp[v]) continue;
        uint4 w = lds16(st + ydst[v]);
        if (yneg[v]) w = make_uint4(w.x ^ NEG, w.y ^ NEG, w.z ^ NEG, w.w ^ NEG);
        sts16(st + yidst[v], w);
      }
    };

    struct Cur {
      int gt, c;
    };
    auto advance = [&](Cur& u) {
      if (++u.c == nchunk) u.c = 0, ++u.gt;
    };
    // plane-wave chunk swept at position c of tile gt (alternating direction)
    auto chunk_of = [&](Cur u) { return (u.gt & 1) ? nchunk - 1 - u.c : u.c; };
    auto load_pos = [&](Cur u) -> int {
      const int G = u.gt * GPT + xg;
      if (u.gt >= ngt || !xok || G >= V.nlf) return -1;
      return (int)mp[(size_t)G * V.nsum_max + chunk_of(u) * VM_I];
    };
    auto issue = [&](Cur u, int stage, int pos) {
      if (u.gt < ngt) {
        const uint32_t st = sbase + (uint32_t)stage * STAGE;
        const __half* src = xsrc + (size_t)(pos >= 0 ? pos : 0) * pstride;
        const uint32_t sz = pos >= 0 ? 16u : 0u;
#pragma unroll
        for (int u4 = 0; u4 < 4; ++u4)
          cp16z(st + xoff + (uint32_t)(u4 >> 1) * XH + (uint32_t)(u4 & 1) * 8192u, src + u4 * V.nbp, sz);
        const int i0 = chunk_of(u) * VM_I;
        const size_t off = (size_t)i0 * pstride;
#pragma unroll
        for (int v = 0; v < YV; ++v) {
          if (!ycp[v]) continue;
          const bool ok = i0 < ylim[v];
          cp16z(st + ydst[v], ok ? ysb[v] + off : ysrc_c, ok ? 16u : 0u);
        }
      }
      cp_commit();
    };

    // accumulator slice: TMEM lane quadrant wq, columns cg CW .. cg CW + CW - 1 of each block
    const int wq = warp & 3, cg = warp >> 2;
    const int row_t = wq * 32 + lane;
    const int eg = row_t / XB, ea = row_t - eg * XB;
    // FP32 sums over the chunks, pairs of columns (packed f32x2 arithmetic)
    constexpr int CH = CW / 2;
    float2 accR[NP][CH], accI[NP][CH];
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
      for (int j = 0; j < CH; ++j) accR[p][j] = accI[p][j] = make_float2(0.f, 0.f);
    float fa[NP];
    auto set_afac = [&](int gt) {
      const int G = gt * GPT + eg;
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        fa[p] = 0.f;
        if (CURRENT && eg < GPT && G < V.nlf) {
          const double* kv = V.ktot + 3 * ik;
          const double* gl = V.Glf + 3 * G;
          const int mu = p == 0 ? V.comp : V.comp2;
          const double qmu = mu == 0 ? V.q0 : (mu == 1 ? V.q1 : V.q2);
          fa[p] = (float)(0.5 * V.Gcar * (qmu + 2.0 * kv[mu] + gl[mu])) * V.a_scale;
        }
      }
    };
    auto consume = [&](int t) -> bool {
      constexpr int NBF = Cfg::NBUF;
      if (!tc::mbar_wait(&done[t % NBF], (uint32_t)((t / NBF) & 1), VM_SPINS)) {
        atomicExch(V.status, 1);
        abort_flag = 1;
        return false;
      }
      tc::tc_fence_after();
      const uint32_t ad = taddr + ((uint32_t)(wq * 32) << 16) + (uint32_t)((t % NBF) * Cfg::N2 + cg * CW);
      float vr[NB][CW], vi[NB][CW];  // Re D, Im D of each column block
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        tmem_ld_n<CW>(ad + b * NBY, vr[b]);
        tmem_ld_n<CW>(ad + NYN + b * NBY, vi[b]);
      }
      tc::tmem_ld_wait();
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&tfree[t % NBF]);
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        const float2 r0 = make_float2(vr[0][2 * j], vr[0][2 * j + 1]);
        const float2 i0 = make_float2(vi[0][2 * j], vi[0][2 * j + 1]);
        if constexpr (CURRENT) {
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float2 f2 = make_float2(fa[p], fa[p]);
            const float2 rp = make_float2(vr[p + 1][2 * j], vr[p + 1][2 * j + 1]);
            const float2 ip = make_float2(vi[p + 1][2 * j], vi[p + 1][2 * j + 1]);
            accR[p][j] = __fadd2_rn(accR[p][j], __ffma2_rn(f2, r0, rp));
            accI[p][j] = __fadd2_rn(accI[p][j], __ffma2_rn(f2, i0, ip));
          }
        } else {
          accR[0][j] = __fadd2_rn(accR[0][j], r0);
          accI[0][j] = __fadd2_rn(accI[0][j], i0);
        }
      }
      return true;
    };
    float amx[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) amx[p] = 0.f;
    const float isign = V.swap ? -V.out_scale : V.out_scale;
    auto write_out = [&](int gt) {
      const int G = gt * GPT + eg;
      if (eg < GPT && G < V.nlf) {
#pragma unroll
        for (int q = 0; q < CW / 4; ++q) {
          int rr[4];  // vertex rows of columns 4 q .. 4 q + 3
          load_rows<4>(ptab + ea * NBY + cg * CW + 4 * q, rr);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int j = 4 * q + i, r = rr[i];
            if (r >= 0) {
#pragma unroll
              for (int p = 0; p < NP; ++p) {
                const float ar = (j & 1) ? accR[p][j >> 1].y : accR[p][j >> 1].x;
                const float ai = (j & 1) ? accI[p][j >> 1].y : accI[p][j >> 1].x;
                const float re = ar * V.out_scale, im = ai * isign;
                (p == 0 ? V.M : V.M2)[(size_t)r * V.nlf + G] = make_float2(re, im);
                amx[p] = fmaxf(amx[p], fmaxf(fabsf(re), fabsf(im)));
              }
            }
          }
        }
      }
#pragma unroll
      for (int p = 0; p < NP; ++p)
#pragma unroll
        for (int j = 0; j < CH; ++j) accR[p][j] = accI[p][j] = make_float2(0.f, 0.f);
    };

    // prologue: chunks 0 .. S-2 in flight.  The Gfast positions of a chunk are
    // loaded two chunks ahead into one of two registers that alternate by
    // chunk parity (the loop below is unrolled by two), so a pending load is
    // never copied between registers.
    Cur ui = {0, 0}, ug = {0, 0};
    int pA = load_pos(ug);
    advance(ug);
    int pB = load_pos(ug);
    advance(ug);
    auto issue_with = [&](int stage, int& R) {
      issue(ui, stage, R);
      advance(ui);
      R = load_pos(ug);
      advance(ug);
    };
#pragma unroll
    for (int s = 0; s < S - 1; ++s) issue_with(s, (s & 1) ? pB : pA);
    cp_wait<S - 2>();
    form(0);
    tc::fence_async_smem();
    __syncwarp();
    if (lane == 0) tc::mbar_arrive(&full[0]);
    set_afac(0);
    Cur uc = {0, 0};   // chunk read back next
    int si = S - 1;    // stage of the next chunk to issue
    int sf = 1 % S;    // stage of chunk j + 1
    bool fail = false;
    auto read_back = [&](int j) -> bool {
      if (!consume(j)) return false;
      if (uc.c == nchunk - 1) {
        write_out(uc.gt);
        set_afac(uc.gt + 1);
      }
      advance(uc);
      return true;
    };
    auto signal = [&](int j) {
      if (j + 1 < total) form(sf);
      tc::fence_async_smem();
      __syncwarp();
      if (lane == 0 && j + 1 < total) tc::mbar_arrive(&full[sf]);
      sf = sf + 1 == S ? 0 : sf + 1;
    };
    // Step j: chunk j + 1 to the MMA warp, chunk j - 1 read back, chunk
    // j + S - 1 issued into the stage of chunk j - 1.
    auto body = [&](int j, int& R) -> bool {
      if constexpr (Cfg::EARLY) {
        // chunk j + 1 (issued S - 2 steps ago) is signalled before this step
        // waits for the MMAs of chunk j - 1, so the MMA warp learns that its
        // operands are in without waiting for that read-back round trip
        cp_wait<S - 3>();
        signal(j);
        if (j >= 1 && !read_back(j - 1)) return false;
        issue_with(si, R);
        si = si + 1 == S ? 0 : si + 1;
      } else {
        // three stages: chunk j + 1 was issued one step ago
        if (j >= 1 && !read_back(j - 1)) return false;
        issue_with(si, R);
        si = si + 1 == S ? 0 : si + 1;
        cp_wait<S - 2>();
        signal(j);
      }
      return !abort_flag;
    };
    // chunk j + S - 1 is issued at step j: its positions are in pA for even
    // j + S - 1, pB for odd
    int& R0 = ((S - 1) & 1) ? pB : pA;
    int& R1 = ((S - 1) & 1) ? pA : pB;
    for (int j = 0; j < total; j += 2) {
      if (!body(j, R0) || (j + 1 < total && !body(j + 1, R1))) {
        fail = true;
        break;
      }
    }
    if (!fail && consume(total - 1)) write_out(ngt - 1);
    cp_wait<0>();
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      float a = amx[p];
      for (int o = 16; o > 0; o >>= 1) a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
      if (lane == 0) atomicMax(V.amax + p, __float_as_uint(a));
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, Cfg::NCOL);
}

// The three-block pass (two Cartesian components) with the worker roles split:
// warps 0-7 read the TMEM accumulators back (two per lane quadrant, 16 of the
// window's columns of each block), warps 8-15 gather and copy the stages and
// signal them, warp 16 issues the MMAs and commits, besides each chunk's
// accumulator, the release of its stage.  The roles advance independently: a
// chunk is signalled as soon as its copies land, a stage is refilled as soon
// as its MMAs are done, an accumulator is freed as soon as it is read back.
// Registers (setmaxnreg, which acts per warpgroup): 256 x 136 (read-back) +
// 256 x 56 (copies) + 32 x 96 (the MMA warp, alone in its warpgroup, keeps
// the launch's count) = 544 x 96, the launch's allocation.
constexpr int VS_CONS = 8, VS_PROD = 8;  // warps
constexpr int VS_REG_CONS = 136, VS_REG_PROD = 56;
static_assert(32 * (VS_CONS * VS_REG_CONS + VS_PROD * VS_REG_PROD + 96) == VM_THREADS * 96, "register split");

template <int NBY>
__global__ void __launch_bounds__(VM_THREADS, 1) k_vertex_mn_split(VtxMnCtx V) {
  using Cfg = VmCfg<NBY, 3>;
  constexpr int NP = 2;  // vertex sets written
  constexpr int S = Cfg::S, NYN = Cfg::NYN, NBF = Cfg::NBUF;
  constexpr uint32_t XH = Cfg::XH, YKG = Cfg::YKG, YLO = Cfg::YLO, STAGE = Cfg::STAGE, N2 = Cfg::N2;
  constexpr int CW = NBY / 2;  // columns of each block per read-back thread
  constexpr int CH = CW / 2;
  static_assert(!Cfg::IMG && Cfg::SW64 && !Cfg::PTAB_SMEM && S >= 4, "three-block layout");

  extern __shared__ unsigned char smraw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  const uint32_t sbase = tc::smem_u32(base);
  int* ptab = V.ptab_g + (size_t)blockIdx.x * 32 * NBY;  // [a][b]: vertex row of the pair, -1 none
  __shared__ uint64_t full[VM_SMAX], sfree[VM_SMAX], done[NBF], tfree[NBF];
  __shared__ uint32_t tslot;
  __shared__ volatile int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int kl = blockIdx.x, ik = V.k0 + kl;
  const long long t0 = V.offsets[kl], t1 = V.offsets[kl + 1];
  if (t1 == t0) return;
  const int* km = V.kmap + 5 * ik;
  const int K1 = km[0], K2 = km[2];
  const int kX = V.swap ? K1 : K2, kY = V.swap ? K2 : K1;
  const int nsum = V.legacy ? V.nsum_legacy : V.npw[kY];
  const int nchunk = (nsum + VM_I - 1) / VM_I;
  const int GPT = V.gpt, XB = V.xb;
  const int ngt = (V.nlf + GPT - 1) / GPT;
  const int total = ngt * nchunk;

  if (warp == 0) {
    tc::tmem_alloc(&tslot, Cfg::NCOL);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      tc::mbar_init(&full[s], VS_PROD);
      tc::mbar_init(&sfree[s], 1);
    }
    for (int b = 0; b < NBF; ++b) {
      tc::mbar_init(&done[b], 1);
      tc::mbar_init(&tfree[b], VS_CONS);
    }
    abort_flag = 0;
    tc::fence_mbar_init();
  }
  for (int e = tid; e < XB * NBY; e += VM_THREADS) ptab[e] = -1;
  __syncthreads();
  for (long long t = t0 + tid; t < t1; t += VM_THREADS) {
    const int nm = V.trans[t].nm;
    const int n = nm & 0xffff, m = nm >> 16;
    const int xa = V.swap ? n : m, yb = V.swap ? m : n;
    if (xa >= V.xo0 && xa < V.xo1 && yb >= V.yo0 && yb < V.yo1)
      ptab[(xa - V.xs) * NBY + (yb - V.ys)] = V.pos_of[t];
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t taddr = tslot;
  auto fail_status = [&]() {
    atomicExch(V.status, 1);
    abort_flag = 1;
  };
  struct Cur {
    int gt, c;
  };
  auto advance = [&](Cur& u) {
    if (++u.c == nchunk) u.c = 0, ++u.gt;
  };
  // plane-wave chunk swept at position c of tile gt (alternating direction)
  auto chunk_of = [&](Cur u) { return (u.gt & 1) ? nchunk - 1 - u.c : u.c; };

  if (warp == VM_WORKERS / 32) {
    // ---------------------------------------------------------------- MMA warp
    if (lane == 0) {
      constexpr uint64_t YG2 = 2 * (YKG >> 4);
      const uint32_t id = tc::idesc_f16_mn(128, (uint32_t)NYN, false);
      const uint32_t idn = tc::idesc_f16_mn(128, (uint32_t)NYN, true);
      const uint64_t dx0 = tc::desc_sw128_mn(sbase, 1024u, 2048u);
      const uint64_t dy0 = tc::desc_sw64_mn(sbase + 2 * XH, Cfg::AB, YKG);
      // Under this kernel's shared-memory load an mbarrier test takes
      // ~150-200 cycles even when the phase is long complete, and the MMAs
      // of a chunk stop issuing when the tensor core's queue is full: so the
      // barriers of chunk t + 1 are tested while the MMAs of chunk t are
      // queued, and only a barrier not yet seen complete is waited for
      // between chunks (the abort flag is read every 16 chunks).
      int last = -1, s = 0, ph = 0;
      bool fnext = false, tnext = false;  // barriers of the next chunk seen complete
      for (int t = 0; t < total; ++t) {
        if ((t & 15) == 0 && abort_flag) break;
        if ((!fnext && !tc::mbar_wait(&full[s], (uint32_t)ph, VM_SPINS)) ||
            (!tnext && t >= NBF && !tc::mbar_wait(&tfree[t % NBF], (uint32_t)((t / NBF - 1) & 1), VM_SPINS))) {
          fail_status();
          break;
        }
        tc::tc_fence_after();
        const int sn = s + 1 == S ? 0 : s + 1;
        const int phn = sn == 0 ? ph ^ 1 : ph;
        const uint64_t so = (uint64_t)(((uint32_t)s * STAGE) >> 4);
        const uint64_t dx = dx0 + so, dy = dy0 + so;
        const uint32_t d = taddr + (uint32_t)((t % NBF) * N2);
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          const uint64_t xh = dx + (uint64_t)(ks * 256), xl = xh + (XH >> 4);
          const uint64_t yh = dy + (uint64_t)ks * YG2, yl = yh + (YLO >> 4);
          const uint32_t acc = ks > 0 ? 1u : 0u;
          tc::mma_bf16(d, xl, yh, id, acc);  // Xl . Yh
          tc::mma_bf16(d, xh, yl, id, 1u);   // + Xh . Yl
          tc::mma_bf16(d, xh, yh, id, 1u);   // + Xh . Yh
          // Im D: K rows of X against the other half of Y's K rows
          const uint64_t ih = dy + (uint64_t)(ks ^ 2) * YG2, il = ih + (YLO >> 4);
          const uint32_t ii = ks < 2 ? idn : id;
          tc::mma_bf16(d + (uint32_t)NYN, xl, ih, ii, acc);
          tc::mma_bf16(d + (uint32_t)NYN, xh, il, ii, 1u);
          tc::mma_bf16(d + (uint32_t)NYN, xh, ih, ii, 1u);
          if (ks == 0) fnext = t + 1 >= total || tc::mbar_test_wait(&full[sn], (uint32_t)phn);
          if (ks == 2)
            tnext = t + 1 < NBF || tc::mbar_test_wait(&tfree[(t + 1) % NBF], (uint32_t)(((t + 1) / NBF - 1) & 1));
        }
        tc::mma_commit(&done[t % NBF]);
        tc::mma_commit(&sfree[s]);
        last = t;
        s = sn;
        ph = phn;
      }
      if (last >= 0) tc::mbar_wait(&done[last % NBF], (uint32_t)((last / NBF) & 1), VM_SPINS);
    }
  } else if (warp < VS_CONS) {
    // ------------------------------------------------------------ read-back warps
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(VS_REG_CONS));
    const int wq = warp & 3, hc = warp >> 2;  // lane quadrant, column half of each block
    const int row_t = wq * 32 + lane;
    const int eg = row_t / XB, ea = row_t - eg * XB;
    float2 accR[NP][CH], accI[NP][CH];
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
      for (int j = 0; j < CH; ++j) accR[p][j] = accI[p][j] = make_float2(0.f, 0.f);
    // a(G) of each vertex set for this thread's local field of tile gt
    auto afac = [&](int gt, float (&f)[NP]) {
      const int G = gt * GPT + eg;
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        f[p] = 0.f;
        if (eg < GPT && G < V.nlf) {
          const double* kv = V.ktot + 3 * ik;
          const double* gl = V.Glf + 3 * G;
          const int mu = p == 0 ? V.comp : V.comp2;
          const double qmu = mu == 0 ? V.q0 : (mu == 1 ? V.q1 : V.q2);
          f[p] = (float)(0.5 * V.Gcar * (qmu + 2.0 * kv[mu] + gl[mu])) * V.a_scale;
        }
      }
    };
    float fa[NP], fn[NP];
    afac(0, fa);
    // acc[p] += fa[p] * D[c] + D[b_p c] over this thread's columns of one part
    auto add_block = [&](const float (&vc)[CW], const float (&vb)[CW], int p, float2 (&acc)[NP][CH]) {
      const float2 f2 = make_float2(fa[p], fa[p]);
#pragma unroll
      for (int j = 0; j < CH; ++j)
        acc[p][j] = __fadd2_rn(acc[p][j], __ffma2_rn(f2, make_float2(vc[2 * j], vc[2 * j + 1]),
                                                     make_float2(vb[2 * j], vb[2 * j + 1])));
    };
    float amx[NP] = {0.f, 0.f};
    // A finished tile's sums wait in TMEM, in the columns past the accumulator
    // ring ([column][p][Re, Im] per thread), and go out a few columns per chunk
    // of the next tile while the read-back warps wait for the MMAs: written
    // all at once they held up the read-back, and with it the MMA warp, for
    // the time of the tile's scattered row stores.
    constexpr uint32_t STASH = (uint32_t)(NBF * N2);
    static_assert(STASH + 8 * CW <= Cfg::NCOL, "stash beyond the TMEM allocation");
    const uint32_t stash = taddr + ((uint32_t)(wq * 32) << 16) + STASH + (uint32_t)(hc * 4 * CW);
    const int* prow = ptab + ea * NBY + hc * CW;  // vertex rows of this thread's columns
    const int dper = nchunk > 1 ? (CW + nchunk - 2) / (nchunk - 1) : CW;  // columns written per chunk
    int sj = CW;     // next stashed column to write (CW: none left)
    int sG = -1;     // local field of the stashed tile (-1: padding row)
    int srow = -1;   // vertex row of column sj
    auto drain = [&](int n) {
#pragma unroll 1
      for (int i = 0; i < n && sj < CW; ++i, ++sj) {
        float v[4];
        tc::tmem_ld4(stash + (uint32_t)(4 * sj), v);
        tc::tmem_ld_wait();
        const int r = srow;
        if (sj + 1 < CW) srow = prow[sj + 1];
        if (sG >= 0 && r >= 0) {
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float re = v[2 * p] * V.out_scale, im = v[2 * p + 1] * V.out_scale;
            (p == 0 ? V.M : V.M2)[(size_t)r * V.nlf + sG] = make_float2(re, im);
            amx[p] = fmaxf(amx[p], fmaxf(fabsf(re), fabsf(im)));
          }
        }
      }
    };
    auto stash_tile = [&](int gt) {
      drain(CW);
#pragma unroll
      for (int j = 0; j < CW; ++j) {
        const int h = j >> 1;
        const bool od = j & 1;
        tc::tmem_st4(stash + (uint32_t)(4 * j), __float_as_uint(od ? accR[0][h].y : accR[0][h].x),
                     __float_as_uint(od ? accI[0][h].y : accI[0][h].x),
                     __float_as_uint(od ? accR[1][h].y : accR[1][h].x),
                     __float_as_uint(od ? accI[1][h].y : accI[1][h].x));
      }
      tc::tmem_st_wait();
#pragma unroll
      for (int p = 0; p < NP; ++p)
#pragma unroll
        for (int j = 0; j < CH; ++j) accR[p][j] = accI[p][j] = make_float2(0.f, 0.f);
      const int G = gt * GPT + eg;
      sG = eg < GPT && G < V.nlf ? G : -1;
      sj = 0;
      srow = prow[0];
    };
    Cur uc = {0, 0};
    bool fail = false;
    for (int t = 0; t < total; ++t) {
      const bool tile_end = uc.c == nchunk - 1;
      if (tile_end) afac(uc.gt + 1, fn);  // loads in flight across the wait
      if (!tc::mbar_wait(&done[t % NBF], (uint32_t)((t / NBF) & 1), VM_SPINS)) {
        fail_status();
        fail = true;
        break;
      }
      tc::tc_fence_after();
      const uint32_t ad = taddr + ((uint32_t)(wq * 32) << 16) + (uint32_t)((t % NBF) * N2 + hc * CW);
      float vc[CW], vb[CW];
#pragma unroll
      for (int part = 0; part < 2; ++part) {
        const uint32_t a = ad + (uint32_t)(part * NYN);
        tmem_ld_n<CW>(a, vc);
        tmem_ld_n<CW>(a + NBY, vb);
        tc::tmem_ld_wait();
        add_block(vc, vb, 0, part == 0 ? accR : accI);
        tmem_ld_n<CW>(a + 2 * NBY, vb);
        tc::tmem_ld_wait();
        add_block(vc, vb, 1, part == 0 ? accR : accI);
      }
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&tfree[t % NBF]);
      if (tile_end) {
        stash_tile(uc.gt);
#pragma unroll
        for (int p = 0; p < NP; ++p) fa[p] = fn[p];
      } else {
        drain(dper);
      }
      advance(uc);
      if (abort_flag) {
        fail = true;
        break;
      }
    }
    drain(CW);
    (void)fail;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      float a = amx[p];
      for (int o = 16; o > 0; o >>= 1) a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
      if (lane == 0) atomicMax(V.amax + p, __float_as_uint(a));
    }
  } else {
    // ------------------------------------------------------------- copy warps
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(VS_REG_PROD));
    const int ptid = tid - 32 * VS_CONS;  // 0 .. 255
    // X copies: plane waves xpw and xpw + 16 of the chunk, rows 8 xj .. 8 xj + 7,
    // the four planes each
    const int xpw = ptid >> 4, xj = ptid & 15;
    const int xrow = 8 * xj, xg = xrow / XB, xb0 = xrow - xg * XB;
    const bool xok = xg < GPT && V.xs + xb0 < V.nbp;
    auto xoff_of = [&](int pw) {
      return (uint32_t)(pw >> 3) * 2048u + (uint32_t)(xj >> 3) * 1024u + (uint32_t)(pw & 7) * 128u +
             ((uint32_t)((xj & 7) ^ (pw & 7)) << 4);
    };
    const uint32_t xoffA = xoff_of(xpw), xoffB = xoff_of(xpw + 16);
    const size_t pstride = (size_t)4 * V.nbp;
    const __half* xsrc = V.planes + (size_t)kX * V.npwx * pstride + V.xs + xb0;
    const int16_t* mp = V.map + (size_t)kl * V.nlf * V.nsum_max + xpw;
    // Y copies: e = ptid + 256 v over 2 halves x 64 K rows x NYN / 8 chunks
    constexpr int YCH = NYN / 8, YE = 128 * YCH, YV = YE / (32 * VS_PROD);
    static_assert(YE % (32 * VS_PROD) == 0, "Y copies per thread");
    const __half* ysrc_c = V.planes + (size_t)kY * V.npwx * pstride;
    const __half* ysrc_b1 = V.ybt + (size_t)kl * V.nsum_max * pstride;
    const __half* ysrc_b2 = V.ybt2 + (size_t)kl * V.nsum_max * pstride;
    uint32_t ydst[YV];
    const __half* ysb[YV];
    int ylim[YV];
#pragma unroll
    for (int v = 0; v < YV; ++v) {
      const int e = ptid + 32 * VS_PROD * v;
      const int line = e / YCH, j = e - line * YCH;
      const int half = line >> 6, kk = line & 63, part = kk >> 5, pw = kk & 31;
      const int col = 8 * j, u = 2 * half + part;
      const int blk = col / NBY;
      const int band = V.ys + col - blk * NBY;
      ydst[v] = 2 * XH + (uint32_t)(kk >> 3) * YKG + (uint32_t)half * YLO + (uint32_t)(col >> 5) * 512u +
                (uint32_t)(kk & 7) * 64u + ((uint32_t)(((col >> 3) & 3) ^ ((kk & 7) >> 1)) << 4);
      const __half* bp = blk == 0 ? ysrc_c : (blk == 1 ? ysrc_b1 : ysrc_b2);
      ysb[v] = bp + (size_t)pw * pstride + (band < V.nbp ? u * V.nbp + band : 0);
      ylim[v] = band < V.nbp ? nsum - pw : 0;
    }
    // Gfast positions of the chunk's two plane waves, -1: none
    auto load_pos = [&](Cur u, int& pa, int& pb) {
      const int G = u.gt * GPT + xg;
      if (u.gt >= ngt || !xok || G >= V.nlf) {
        pa = pb = -1;
        return;
      }
      const int16_t* q = mp + (size_t)G * V.nsum_max + chunk_of(u) * VM_I;
      pa = (int)q[0];
      pb = (int)q[16];
    };
    auto issue = [&](Cur u, int stage, int pa, int pb) {
      if (u.gt < ngt) {
        const uint32_t st = sbase + (uint32_t)stage * STAGE;
        const __half* sa = xsrc + (size_t)(pa >= 0 ? pa : 0) * pstride;
        const __half* sb = xsrc + (size_t)(pb >= 0 ? pb : 0) * pstride;
        const uint32_t za = pa >= 0 ? 16u : 0u, zb = pb >= 0 ? 16u : 0u;
#pragma unroll
        for (int u4 = 0; u4 < 4; ++u4) {
          const uint32_t o = (uint32_t)(u4 >> 1) * XH + (uint32_t)(u4 & 1) * 8192u;
          cp16z(st + xoffA + o, sa + u4 * V.nbp, za);
          cp16z(st + xoffB + o, sb + u4 * V.nbp, zb);
        }
        const int i0 = chunk_of(u) * VM_I;
        const size_t off = (size_t)i0 * pstride;
#pragma unroll
        for (int v = 0; v < YV; ++v) {
          const bool ok = i0 < ylim[v];
          cp16z(st + ydst[v], ok ? ysb[v] + off : ysrc_c, ok ? 16u : 0u);
        }
      }
      cp_commit();
    };
    auto signal = [&](int s) {
      tc::fence_async_smem();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&full[s]);
    };
    // chunks 0 .. S - 2 in flight, positions one chunk ahead
    Cur ui = {0, 0};
    int pa = 0, pb = 0, na = 0, nb = 0;
    load_pos(ui, pa, pb);
#pragma unroll 1
    for (int s = 0; s < S - 1; ++s) {
      Cur un = ui;
      advance(un);
      load_pos(un, na, nb);
      issue(ui, s, pa, pb);
      ui = un;
      pa = na;
      pb = nb;
    }
    cp_wait<S - 2>();
    signal(0);
    // step j: chunk j + 1 (issued S - 2 steps ago) signalled, then chunk
    // j + S - 1 issued into the stage of chunk j - 1 once its MMAs are done
    for (int j = 0; j < total; ++j) {
      cp_wait<S - 3>();
      if (j + 1 < total) signal((j + 1) % S);
      if (j >= 1 && !tc::mbar_wait(&sfree[(j - 1) % S], (uint32_t)(((j - 1) / S) & 1), VM_SPINS)) {
        fail_status();
        break;
      }
      Cur un = ui;
      advance(un);
      load_pos(un, na, nb);
      issue(ui, (j + S - 1) % S, pa, pb);
      ui = un;
      pa = na;
      pb = nb;
      if (abort_flag) break;
    }
    cp_wait<0>();
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, Cfg::NCOL);
}

// b(i) c of every FBZ k-point of the launch, split like the coefficient planes:
// ybt[k_local][i][plane][band], b(i) = Gcar (R1 G1_i)_mu sB / 2^14 (zero beyond
// nsum), c the planes of K1; (h + l) b is split again into fp16 hi + lo.  With
// comp2 >= 0 the same for the second component into ybt2, from the same loads.
struct YbtCtx {
  const int* kmap;
  const double* G;
  const double* Rcart;
  const int* gidx;
  const int* npw;
  const __half* planes;
  __half* ybt;
  __half* ybt2;
  int k0, nk, npwx, nbp, nsum_max, legacy, nsum_legacy, comp, comp2;
  double Gcar;
  float sB;
};

// (h + l) b for the eight bands of p[], split into fp16 hi + lo planes
__device__ __forceinline__ void ybt_split(const uint4* p, float b, __half* out, int nbp) {
  uint4 o[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    // bands 2q, 2q + 1 of the group: re = re_hi + re_lo, im = im_hi + im_lo
    const float2 rh = __half22float2(reinterpret_cast<const __half2*>(&p[0])[q]);
    const float2 ih = __half22float2(reinterpret_cast<const __half2*>(&p[1])[q]);
    const float2 rl = __half22float2(reinterpret_cast<const __half2*>(&p[2])[q]);
    const float2 il = __half22float2(reinterpret_cast<const __half2*>(&p[3])[q]);
    const float2 re = make_float2((rh.x + rl.x) * b, (rh.y + rl.y) * b);
    const float2 im = make_float2((ih.x + il.x) * b, (ih.y + il.y) * b);
    const __half2 reh = __floats2half2_rn(re.x, re.y), imh = __floats2half2_rn(im.x, im.y);
    const float2 rehf = __half22float2(reh), imhf = __half22float2(imh);
    const __half2 rel = __floats2half2_rn(re.x - rehf.x, re.y - rehf.y);
    const __half2 iml = __floats2half2_rn(im.x - imhf.x, im.y - imhf.y);
    reinterpret_cast<__half2*>(&o[0])[q] = reh;
    reinterpret_cast<__half2*>(&o[1])[q] = imh;
    reinterpret_cast<__half2*>(&o[2])[q] = rel;
    reinterpret_cast<__half2*>(&o[3])[q] = iml;
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) *reinterpret_cast<uint4*>(out + u * nbp) = o[u];
}

// One thread per (k-point, plane wave, 8-band group): 16-byte loads of the four
// coefficient planes and 16-byte stores of the four b(i) c planes (per component).
__global__ void k_vtx_ybt(YbtCtx Y) {
  const int ng = Y.nbp / 8;
  const size_t n = (size_t)Y.nk * Y.nsum_max * ng;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int g = (int)(e % ng);
    const size_t r = e / ng;
    const int i = (int)(r % Y.nsum_max), kl = (int)(r / Y.nsum_max);
    const int* km = Y.kmap + 5 * (Y.k0 + kl);
    const int K1 = km[0];
    const int nsum = Y.legacy ? Y.nsum_legacy : Y.npw[K1];
    float b = 0.f, b2 = 0.f;
    if (i < nsum) {
      const double* g1 = Y.G + 3 * Y.gidx[(size_t)K1 * Y.npwx + i];
      const double* R = Y.Rcart + 9 * km[1] + 3 * Y.comp;
      b = (float)(Y.Gcar * (R[0] * g1[0] + R[1] * g1[1] + R[2] * g1[2])) * Y.sB * (1.0f / 16384.0f);
      if (Y.comp2 >= 0) {
        const double* R2 = Y.Rcart + 9 * km[1] + 3 * Y.comp2;
        b2 = (float)(Y.Gcar * (R2[0] * g1[0] + R2[1] * g1[1] + R2[2] * g1[2])) * Y.sB * (1.0f / 16384.0f);
      }
    }
    const __half* c = Y.planes + ((size_t)K1 * Y.npwx + (i < nsum ? i : 0)) * 4 * Y.nbp + 8 * g;
    uint4 p[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) p[u] = __ldg(reinterpret_cast<const uint4*>(c + u * Y.nbp));
    ybt_split(p, b, Y.ybt + r * 4 * Y.nbp + 8 * g, Y.nbp);
    if (Y.comp2 >= 0) ybt_split(p, b2, Y.ybt2 + r * 4 * Y.nbp + 8 * g, Y.nbp);
  }
}

template <int NBY, int NB>
static int launch_vmn(rpa_ctx* c, const VtxMnCtx& V, int nk) {
  using Cfg = VmCfg<NBY, NB>;
  auto kern = k_vertex_mn<NBY, NB>;
  RPA_CUDA(c, allow_dynamic_smem(kern, c->device));
  kern<<<nk, VM_THREADS, Cfg::SMEM, c->stream>>>(V);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

template <int NBY>
static int launch_vmn_split(rpa_ctx* c, const VtxMnCtx& V, int nk) {
  using Cfg = VmCfg<NBY, 3>;
  auto kern = k_vertex_mn_split<NBY>;
  RPA_CUDA(c, allow_dynamic_smem(kern, c->device));
  kern<<<nk, VM_THREADS, Cfg::SMEM, c->stream>>>(V);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

// nb: column blocks of Y (1 charge, 2 current, 3 current with two components)
static int launch_vmn_nby(rpa_ctx* c, const VtxMnCtx& V, int nk, int nby, int nb) {
  if (nb == 1) {
    if (nby == 16) return launch_vmn<16, 1>(c, V, nk);
    if (nby == 32) return launch_vmn<32, 1>(c, V, nk);
    if (nby == 48) return launch_vmn<48, 1>(c, V, nk);
    if (nby == 64) return launch_vmn<64, 1>(c, V, nk);
  } else if (nb == 2) {
    if (nby == 16) return launch_vmn<16, 2>(c, V, nk);
    if (nby == 32) return launch_vmn<32, 2>(c, V, nk);
  } else if (nb == 3) {
    if (nby == 16) return launch_vmn_split<16>(c, V, nk);
    if (nby == 32) return launch_vmn_split<32>(c, V, nk);
  }
  return fail(c, RPA_EINVAL, "vertices: no kernel for a %d-band window with %d column blocks", nby, nb);
}

// One launch per pair of band windows: gathered bands [x0, x1) in windows of
// 32 starting on multiples of 8, sequential bands [y0, y1) in windows of at most
// ymax (multiples of 16 wide, starting on a multiple of 8; the Y tile spans at
// most 128 columns so that three stages fit).
static int launch_windows_mn(rpa_ctx* c, VtxMnCtx V, int nk, int x0, int x1, int y0, int y1, int ymax, int nb) {
  const int ys0 = y0 & ~7, span = y1 - ys0;
  const int nyw = (span + ymax - 1) / ymax;
  const int W = ((span + nyw - 1) / nyw + 15) / 16 * 16;
  for (int ws = x0 & ~7; ws < x1; ws += 32) {
    V.xs = ws;
    V.xo0 = std::max(x0, ws);
    V.xo1 = std::min(x1, ws + 32);
    V.xb = (V.xo1 - ws + 7) / 8 * 8;
    V.gpt = 128 / V.xb;
    for (int w = 0; w < nyw; ++w) {
      V.ys = ys0 + w * W;
      V.yo0 = std::max(y0, V.ys);
      V.yo1 = std::min(y1, V.ys + W);
      if (V.yo1 <= V.yo0) continue;
      RPA_TRY(launch_vmn_nby(c, V, nk, W, nb));
    }
  }
  return RPA_OK;
}

static double pow2_floor_m(double x) { return std::ldexp(1.0, (int)std::floor(std::log2(x))); }

// Mixed-path vertices of the FBZ k-points [k0, k0+nk) with MN-major operands.
// Leaves *used false when the plane-wave count does not fit the int16 map
// positions or the band count the int16 pair table.  Current vertices of the
// yz / zy pair go to Mf and Mf2 in one pass; with extra_pol (RPA_POL_XX / YY /
// ZZ, not the call's own) a single-component polarisation also gets the
// vertices of extra_pol into Mf2, from the same pass.
int vertices_mn(rpa_ctx* c, const Chi0Plan& P, int k0, int nk, long long n_trans, const int* pos_of, float2* Mf,
                float2* Mf2, unsigned* amax, bool* used, int extra_pol) {
  *used = false;
  if (n_trans == 0) return RPA_OK;
  if (c->npwx > 32767 || c->nbnd > 181 || c->d_cpl.p == nullptr) return RPA_OK;
  const bool current = P.mode == RPA_MODE_CURRENT;
  const bool two = current && (P.pol == RPA_POL_YZ || P.pol == RPA_POL_ZY);
  // gathered side of charge vertices: the tuned choice, else the side with fewer bands
  const int want_swap = c->vt_cur.swap >= 0 ? c->vt_cur.swap : (P.nocc < c->nbnd - P.nocc ? 1 : 0);
  const bool swap = !current && !c->legacy && want_swap == 1;
  const int ymax_cur = c->vt_cur.ymax > 0 ? std::min(c->vt_cur.ymax, 32) : 32;
  const int ymax_chg = c->vt_cur.ymax > 0 ? std::min(c->vt_cur.ymax, 64) : 64;
  int x0, x1, y0, y1;
  if (current) {
    x0 = 0, x1 = c->nbnd, y0 = 0, y1 = c->nbnd;
  } else if (swap) {
    x0 = 0, x1 = P.nocc, y0 = P.nocc, y1 = c->nbnd;
  } else {
    x0 = P.nocc, x1 = c->nbnd, y0 = 0, y1 = P.nocc;
  }
  if (x1 <= x0 || y1 <= y0) return RPA_OK;
  // sequential side: plane waves of K1 (K2 when swapped)
  int nsum_max = 0;
  for (int i = 0; i < nk; ++i) {
    const int* km = &c->h_kmap[5 * (size_t)(k0 + i)];
    nsum_max = std::max(nsum_max, c->legacy ? P.nsum_legacy : c->h_npw[swap ? km[2] : km[0]]);
  }
  nsum_max = (nsum_max + VM_I - 1) / VM_I * VM_I;
  const int16_t* map;
  if (swap) {
    const size_t gbytes = (size_t)nk * c->nlf * nsum_max * sizeof(int16_t);
    if (!(c->ginv_valid && c->ginv_k0 == k0 && c->ginv_nk == nk && c->ginv_nsum == nsum_max)) {
      RPA_TRY(ensure(c, c->d_ginv, gbytes));
      RPA_TRY(build_ginv(c, k0, nk, nsum_max, c->d_ginv.as<int16_t>()));
      c->ginv_valid = true;
      c->ginv_k0 = k0;
      c->ginv_nk = nk;
      c->ginv_nsum = nsum_max;
    }
    map = c->d_ginv.as<int16_t>();
  } else {
    const size_t gbytes = (size_t)nk * c->nlf * nsum_max * sizeof(int16_t);
    if (!(c->gmap_valid && c->gmap_k0 == k0 && c->gmap_nk == nk && c->gmap_nsum == nsum_max &&
          c->gmap_legacy_n == P.nsum_legacy)) {
      RPA_TRY(ensure(c, c->d_gmap, gbytes));
      RPA_TRY(build_gmap(c, k0, nk, nsum_max, c->d_gmap.as<int16_t>(), P.nsum_legacy));
      c->gmap_valid = true;
      c->gmap_k0 = k0;
      c->gmap_nk = nk;
      c->gmap_nsum = nsum_max;
      c->gmap_legacy_n = P.nsum_legacy;
    }
    map = c->d_gmap.as<int16_t>();
  }
  VtxMnCtx V;
  V.kmap = c->d_kmap.as<int>();
  V.ktot = c->d_ktot.as<double>();
  V.Glf = c->d_Glf.as<double>();
  V.npw = c->d_npw.as<int>();
  V.planes = c->d_cpl.as<__half>();
  V.ybt = V.ybt2 = nullptr;
  V.M2 = nullptr;
  V.ptab_g = nullptr;
  V.comp2 = 0;
  V.map = map;
  V.trans = c->d_trans.as<Trans>();
  V.offsets = c->d_offsets.as<long long>();
  V.pos_of = pos_of;
  V.status = c->d_flags.as<int>() + 3;
  V.k0 = k0;
  V.nlf = c->nlf;
  V.npwx = c->npwx;
  V.nbp = c->nbp;
  V.nsum_max = nsum_max;
  V.legacy = c->legacy ? 1 : 0;
  V.nsum_legacy = P.nsum_legacy;
  V.swap = swap ? 1 : 0;
  V.q0 = c->q[0];
  V.q1 = c->q[1];
  V.q2 = c->q[2];
  V.Gcar = P.Gcar;
  if (!current) {
    V.comp = V.comp2 = 0;
    V.a_scale = 0.0f;
    V.out_scale = (float)(1.0 / (16384.0 * 16384.0));
    V.M = V.M2 = Mf;
    V.ybt2 = nullptr;
    V.amax = amax;
    *used = true;
    return launch_windows_mn(c, V, nk, x0, x1, y0, y1, ymax_chg, 1);
  }
  // current vertices: |C| <= 1 (orthonormal bands), |b(i)| <= Gcar max|G|
  double gmax = 0.0;
  for (size_t g = 0; g < c->h_G.size() / 3; ++g) {
    const double* v = &c->h_G[3 * g];
    gmax = std::max(gmax, std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
  }
  const double bmax = std::max(P.Gcar * gmax, 1e-30);
  const float sB = (float)(16384.0 / pow2_floor_m(bmax * 1.5));
  V.a_scale = sB / 16384.0f;
  V.out_scale = (float)(1.0 / (16384.0 * (double)sB));
  int comps[2];
  switch (P.pol) {
    case RPA_POL_XX: comps[0] = comps[1] = 0; break;
    case RPA_POL_YY: comps[0] = comps[1] = 1; break;
    case RPA_POL_ZZ: comps[0] = comps[1] = 2; break;
    case RPA_POL_YZ: comps[0] = 1; comps[1] = 2; break;
    default: comps[0] = 2; comps[1] = 1; break;
  }
  bool pair = two;
  if (!two && extra_pol >= 0) {
    comps[1] = extra_pol == RPA_POL_XX ? 0 : (extra_pol == RPA_POL_YY ? 1 : 2);
    pair = true;
  }
  if (pair) {
    RPA_TRY(ensure(c, c->d_ptab, sizeof(int) * (size_t)nk * 32 * 32));
    V.ptab_g = c->d_ptab.as<int>();
  }
  const size_t ybt_n = (size_t)nk * nsum_max * 4 * c->nbp;
  RPA_TRY(ensure(c, c->d_ybt, sizeof(__half) * ybt_n * (pair ? 2 : 1)));
  V.ybt = c->d_ybt.as<__half>();
  V.ybt2 = pair ? V.ybt + ybt_n : nullptr;
  YbtCtx Y;
  Y.kmap = V.kmap;
  Y.G = c->d_G.as<double>();
  Y.Rcart = c->d_Rcart.as<double>();
  Y.gidx = c->d_gidx.as<int>();
  Y.npw = V.npw;
  Y.planes = V.planes;
  Y.ybt = c->d_ybt.as<__half>();
  Y.k0 = k0;
  Y.nk = nk;
  Y.npwx = c->npwx;
  Y.nbp = c->nbp;
  Y.nsum_max = nsum_max;
  Y.legacy = V.legacy;
  Y.nsum_legacy = P.nsum_legacy;
  Y.Gcar = P.Gcar;
  Y.sB = sB;
  Y.ybt2 = const_cast<__half*>(V.ybt2);
  V.comp = Y.comp = comps[0];
  V.comp2 = comps[1];
  Y.comp2 = pair ? comps[1] : -1;
  V.M = Mf;
  V.M2 = pair ? Mf2 : Mf;
  V.amax = amax;
  k_vtx_ybt<<<2 * 152 * 8, 256, 0, c->stream>>>(Y);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  RPA_TRY(launch_windows_mn(c, V, nk, x0, x1, y0, y1, ymax_cur, pair ? 3 : 2));
  *used = true;
  return RPA_OK;
}

}  // namespace rpa
