// k_vertex_tc.cu -- plane-wave vertices on the tcgen05 tensor cores (mixed path).
//
// Same vertices as k_vertex.cu (genMnmK1K2, Sloss.f90:883-952; genStrujniVrhovi,
// Optabs.f90:1354-1472), written per FBZ k-point as a GEMM over the plane
// waves i of K1:
//     M_nm(G) = sum_i conj(C1[n,i]) * f(G,i) * C2[m, Gfast(G,i)]
// rows = (G, m) pairs, 128 / mcount local fields per 128-row tile; columns =
// bands n of K1; K = plane waves, 32 per chunk, each contributing its (re, im)
// pair as two adjacent K elements:
//     X((G,m), i) = ( Re y,  Im y ),   y = C2[m, Gfast(G,i)]
//     Y(n, i)     = ( Re c,  Im c )  ->  D((G,m), n)      = Re sum conj(c) y
//     Y(NB+n, i)  = ( -Im c, Re c )  ->  D((G,m), NB + n) = Im sum conj(c) y
// The current factor of Optabs separates, f(G,i) = a(G) + b(i) with
// a(G) = 0.5 Gcar (q + 2k + Glf_G)_mu and b(i) = Gcar (R1 G1_i)_mu, so b(i) goes
// into a second column block of the band operand (c -> b(i) c) and a(G) is
// applied per row when the accumulator is read:
//     M = a(G) * D[Y] + D[b Y]
// The coefficients are stored once, scaled by 2^14, as packed fp16 hi + lo
// words {re_hi | im_hi << 16, re_lo | im_lo << 16}.  With the (re, im) pair
// order the gathered operand X is those words unchanged, so cp.async copies
// them from global memory straight into the 128-byte-swizzled hi and lo tiles
// through a ring of S shared-memory stages (zero-filled where Gfast has no
// match); the Re rows of Y arrive the same way.  Threads only form the Im rows
// and the b(i) rows.  D = Xh Yl + Xl Yh + Xh Yh (small products first); each
// chunk accumulates in a fresh TMEM buffer (two, ping-pong) that is added to
// FP32 registers, as in k_accum_tc.cu.  Inside a chunk the K slot s holds plane
// wave 8 (s % 4) + s / 4, which makes both the gathers (4 plane waves x 8
// bands per warp instruction) and the shared-memory writes conflict-free.

#include <cuda_fp16.h>

#include <cmath>

#include "rpa_internal.cuh"
#include "tc05.cuh"

namespace rpa {

int build_gmap(rpa_ctx* c, int k0, int nk, int nsum_max, int16_t* gmap, int nsum_legacy);

struct VtxTcCtx {
  const int* kmap;
  const double* ktot;
  const double* G;        // Cartesian G list
  const double* Rcart;    // [48][9]
  const int* gidx;        // [kibz][npwx]
  const int* npw;
  const double* Glf;      // [nlf][3]
  const uint2* coeffs;    // split fp16 coefficients x 2^14 [kibz][npwx][nbnd]
  const int16_t* gmap;    // [k_local][nlf][nsum_max]
  const float* btab;      // b(i) sB / 2^14, [k_local][nsum_max] (current vertices)
  const Trans* trans;
  const long long* offsets;
  const int* pos_of;
  float2* M;
  unsigned* amax;
  int* status;
  int k0, nlf, npwx, nbnd, legacy, nsum_legacy, nsum_max;
  int m0, mcount, n0, ncount, gpt;
  int comp;               // Cartesian component of the current vertex
  double q0, q1, q2, Gcar;
  float sB;               // scale of the b(i) Y block (X and Y carry the 2^14 of the split coefficients)
  float out_scale;        // 2^-28 (charge) or 1 / (2^14 sB) (current)
  float a_scale;          // sB / 2^14: a(G) D[Y] in units of D[b Y]
};

constexpr int VT_I = 32;          // plane waves per chunk (K = 64)
constexpr int VT_THREADS = 512;   // 16 warps: 4 TMEM lane quadrants x 4 column groups
constexpr uint32_t VT_SPINS = 1u << 16;  // suspending polls: about 1.3 s at most
constexpr int VT_SMEM_MAX = 232448 - 4608;  // dynamic shared memory left beside the static tables

template <int NB, bool CURRENT>
struct VtCfg {
  static constexpr int NY = CURRENT ? 2 : 1;  // column blocks: c, b c
  static constexpr int N = NY * 2 * NB;
  static constexpr uint32_t X_BYTES = 128 * 128, Y_BYTES = N * 128;
  static constexpr uint32_t B_OFF = 2 * X_BYTES + 2 * Y_BYTES;                 // b(i) of the chunk, 32 floats
  static constexpr uint32_t STAGE = (B_OFF + (CURRENT ? 128 : 0) + 1023) / 1024 * 1024;
  static constexpr int S0 = (VT_SMEM_MAX - 1024) / (int)STAGE;
  static constexpr int S = S0 > 5 ? 5 : S0;                                      // ring depth
  static constexpr uint32_t NCOL = 2 * N <= 32 ? 32 : 2 * N <= 64 ? 64 : 2 * N <= 128 ? 128 : 256;
  static constexpr uint32_t BUF = NCOL / 2;  // TMEM column stride of the two buffers
  static constexpr int CW = NB / 2;          // accumulator columns per thread per block
  static constexpr size_t SMEM = (size_t)S * STAGE + 1024;
};

// plane wave (within the chunk) held by K slot s
__device__ __forceinline__ int vt_pw(int s) { return 8 * (s & 3) + (s >> 2); }

// byte offset of the 4-byte K slot s of row r in a 128-byte-swizzled tile
__device__ __forceinline__ uint32_t vt_off(int r, int s) {
  return (uint32_t)r * 128u + ((uint32_t)((s >> 2) ^ (r & 7)) << 4) + (uint32_t)(s & 3) * 4u;
}

__device__ __forceinline__ void cp_async4(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory");
}

// (re, im) fp16 pair -> (-im, re), exactly
__device__ __forceinline__ uint32_t negswap(uint32_t w) { return __byte_perm(w, 0, 0x1032) ^ 0x00008000u; }

__device__ __forceinline__ uint32_t pack_h2(__half2 h) { return *reinterpret_cast<uint32_t*>(&h); }

template <int CW>
__device__ __forceinline__ void tmem_ld_cw(uint32_t addr, float* v) {
  if constexpr (CW == 16) tc::tmem_ld16(addr, v);
  else if constexpr (CW == 8) tc::tmem_ld8(addr, v);
  else tc::tmem_ld4(addr, v);
}

// One CTA per FBZ k-point.  NB: bands n per tile (8, 16 or 32).
template <int NB, bool CURRENT>
__global__ void __launch_bounds__(VT_THREADS, 1) k_vertex_tc(VtxTcCtx V) {
  using Cfg = VtCfg<NB, CURRENT>;
  constexpr int NY = Cfg::NY, N = Cfg::N, CW = Cfg::CW, S = Cfg::S;
  constexpr uint32_t STAGE = Cfg::STAGE, X_BYTES = Cfg::X_BYTES, Y_BYTES = Cfg::Y_BYTES;
  static_assert(S >= 3, "shared-memory ring too shallow");

  extern __shared__ unsigned char smraw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  const uint32_t sbase = tc::smem_u32(base);
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tslot;
  __shared__ int ptab[32][32];  // sorted vertex row of (n - n0, m - m0), -1 if none

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int kl = blockIdx.x, ik = V.k0 + kl;
  const long long t0 = V.offsets[kl], t1 = V.offsets[kl + 1];
  if (t1 == t0) return;
  const int* km = V.kmap + 5 * ik;
  const int K1 = km[0], K2 = km[2];
  const int nsum = V.legacy ? V.nsum_legacy : V.npw[K1];
  const int nchunk = (nsum + VT_I - 1) / VT_I;
  const int GPT = V.gpt, mcount = V.mcount;
  const int ngt = (V.nlf + GPT - 1) / GPT;
  const int total = ngt * nchunk;

  if (warp == 0) {
    tc::tmem_alloc(&tslot, Cfg::NCOL);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    tc::fence_mbar_init();
  }
  for (int e = tid; e < 32 * 32; e += VT_THREADS) (&ptab[0][0])[e] = -1;
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  for (long long t = t0 + tid; t < t1; t += VT_THREADS) {
    int nm = V.trans[t].nm;
    int n = (nm & 0xffff) - V.n0, m = (nm >> 16) - V.m0;
    if (n >= 0 && n < V.ncount && m >= 0 && m < mcount) ptab[n][m] = V.pos_of[t];
  }
  const uint32_t taddr = tslot;
  const uint32_t idesc = tc::idesc_bf16(128, N, true);
  const int16_t* gm = V.gmap + (size_t)kl * V.nlf * V.nsum_max;
  const float* bt = CURRENT ? V.btab + (size_t)kl * V.nsum_max : nullptr;

  // gather task of this thread: X row xr, plane waves 8 xp .. 8 xp + 7 -> K slots xp + 4 j
  const int xr = 8 * warp + (lane >> 2), xp = lane & 3;
  const int xgl = xr / mcount, xm = xr - xgl * mcount;
  const bool xrow = xgl < GPT;
  const uint2* C2 = V.coeffs + (size_t)K2 * V.npwx * V.nbnd + V.m0 + xm;
  const uint2* C1 = V.coeffs + (size_t)K1 * V.npwx * V.nbnd + V.n0;

  // band-operand elements of this thread: (n, K slot) pairs e = tid + VT_THREADS j
  constexpr int YJ = (NB * 32 + VT_THREADS - 1) / VT_THREADS;
  int yn[YJ], ypw[YJ];
  uint32_t yoff[YJ], yoffi[YJ];
#pragma unroll
  for (int j = 0; j < YJ; ++j) {
    const int e = tid + VT_THREADS * j, blk = e >> 5, l = e & 31;
    const int n = 8 * (blk % (NB / 8)) + (l >> 2), sl = 4 * (blk / (NB / 8)) + (l & 3);
    yn[j] = e < NB * 32 ? n : -1;
    ypw[j] = vt_pw(sl);
    yoff[j] = vt_off(n, sl);
    yoffi[j] = vt_off(NB + n, sl);
  }
  uint32_t xoff[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) xoff[j] = vt_off(xr, xp + 4 * j);

  // (local-field tile, chunk) of a running chunk index, advanced without division
  struct Cur {
    int gt, c;
  };
  auto advance = [&](Cur& u) {
    if (++u.c == nchunk) u.c = 0, ++u.gt;
  };
  auto load_gm = [&](Cur u) -> uint4 {
    uint4 g = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
    const int G = u.gt * GPT + xgl;
    if (u.gt < ngt && xrow && G < V.nlf)
      g = *reinterpret_cast<const uint4*>(gm + (size_t)G * V.nsum_max + u.c * VT_I + xp * 8);
    return g;
  };
  // chunk u -> stage st: X tiles, Re rows of Y, b(i); always one commit group
  auto issue = [&](Cur u, int stage, uint4 g) {
    if (u.gt < ngt) {
      const uint32_t st = sbase + (uint32_t)stage * STAGE;
      const int i0 = u.c * VT_I;
      const uint32_t w[4] = {g.x, g.y, g.z, g.w};
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int pos = (int)(int16_t)(uint16_t)(w[j >> 1] >> ((j & 1) * 16));
        const uint2* src = C2 + (pos >= 0 ? pos : 0) * V.nbnd;
        const uint32_t sz = pos >= 0 ? 4u : 0u;
        cp_async4(st + xoff[j], &src->x, sz);
        cp_async4(st + X_BYTES + xoff[j], &src->y, sz);
      }
#pragma unroll
      for (int j = 0; j < YJ; ++j) {
        if (yn[j] < 0) continue;
        const int i = i0 + ypw[j];
        const bool ok = yn[j] < V.ncount && i < nsum;
        const uint2* src = C1 + (ok ? i * V.nbnd + yn[j] : 0);
        cp_async4(st + 2 * X_BYTES + yoff[j], &src->x, ok ? 4u : 0u);
        cp_async4(st + 2 * X_BYTES + Y_BYTES + yoff[j], &src->y, ok ? 4u : 0u);
      }
      if (CURRENT && tid < 8) cp_async16(st + Cfg::B_OFF + 16 * tid, bt + i0 + 4 * tid);
    }
    cp_async_commit();
  };
  // Im rows of Y (and the b(i) block) of the chunk in a stage, from its Re rows
  auto form = [&](int stage) {
    unsigned char* st = base + (size_t)stage * STAGE;
    unsigned char* yh = st + 2 * X_BYTES;
    unsigned char* yl = yh + Y_BYTES;
    const float* bs = reinterpret_cast<const float*>(st + Cfg::B_OFF);
#pragma unroll
    for (int j = 0; j < YJ; ++j) {
      if (yn[j] < 0) continue;
      const uint32_t wh = *reinterpret_cast<const uint32_t*>(yh + yoff[j]);
      const uint32_t wl = *reinterpret_cast<const uint32_t*>(yl + yoff[j]);
      *reinterpret_cast<uint32_t*>(yh + yoffi[j]) = negswap(wh);
      *reinterpret_cast<uint32_t*>(yl + yoffi[j]) = negswap(wl);
      if (CURRENT) {
        const float b = bs[ypw[j]];
        const float2 h = __half22float2(*reinterpret_cast<const __half2*>(&wh));
        const float2 lo = __half22float2(*reinterpret_cast<const __half2*>(&wl));
        const float re = (h.x + lo.x) * b, im = (h.y + lo.y) * b;
        const __half2 hh = __floats2half2_rn(re, im);
        const float2 hf = __half22float2(hh);
        const __half2 ll = __floats2half2_rn(re - hf.x, im - hf.y);
        const uint32_t bh = pack_h2(hh), bl = pack_h2(ll);
        const uint32_t ob = yoff[j] + 2 * NB * 128, obi = yoffi[j] + 2 * NB * 128;
        *reinterpret_cast<uint32_t*>(yh + ob) = bh;
        *reinterpret_cast<uint32_t*>(yl + ob) = bl;
        *reinterpret_cast<uint32_t*>(yh + obi) = negswap(bh);
        *reinterpret_cast<uint32_t*>(yl + obi) = negswap(bl);
      }
    }
  };

  // accumulator slice of this thread: TMEM lane quadrant wq, column group cg
  const int wq = warp & 3, cg = warp >> 2;
  const int row_t = wq * 32 + lane;
  const int egl = row_t / mcount, em = row_t - egl * mcount;
  float acc[CW];
#pragma unroll
  for (int j = 0; j < CW; ++j) acc[j] = 0.f;
  float fa = 0.f;
  auto set_afac = [&](int gt) {
    const int G = gt * GPT + egl;
    fa = 0.f;
    if (CURRENT && egl < GPT && G < V.nlf) {
      const double* kv = V.ktot + 3 * ik;
      const double* gl = V.Glf + 3 * G;
      const int mu = V.comp;
      const double qmu = mu == 0 ? V.q0 : (mu == 1 ? V.q1 : V.q2);
      fa = (float)(0.5 * V.Gcar * (qmu + 2.0 * kv[mu] + gl[mu])) * V.a_scale;
    }
  };
  auto consume = [&](int buf) {
    const uint32_t ad = taddr + ((uint32_t)(wq * 32) << 16) + (uint32_t)(buf * Cfg::BUF + cg * CW);
    float v[NY][CW];
#pragma unroll
    for (int b = 0; b < NY; ++b) tmem_ld_cw<CW>(ad + b * 2 * NB, v[b]);
    tc::tmem_ld_wait();
#pragma unroll
    for (int j = 0; j < CW; ++j) {
      if (CURRENT) acc[j] += fmaf(fa, v[0][j], v[NY - 1][j]);
      else acc[j] += v[0][j];
    }
  };
  float amx = 0.f;
  auto write_out = [&](int gt) {
    const int G = gt * GPT + egl;
    if (egl < GPT && G < V.nlf) {
      const int part = cg >> 1;
#pragma unroll
      for (int j = 0; j < CW; ++j) {
        const int n = (cg & 1) * CW + j;
        const int r = n < V.ncount ? ptab[n][em] : -1;
        if (r >= 0) {
          const float v = acc[j] * V.out_scale;
          reinterpret_cast<float*>(V.M + (size_t)r * V.nlf + G)[part] = v;
          amx = fmaxf(amx, fabsf(v));
        }
      }
    }
#pragma unroll
    for (int j = 0; j < CW; ++j) acc[j] = 0.f;
  };

  // prologue: chunks 0 .. S-2 in flight, positions of S-1 and S in registers
  Cur ui = {0, 0};  // next chunk to issue
  for (int j = 0; j < S - 1; ++j) {
    issue(ui, j, load_gm(ui));
    advance(ui);
  }
  Cur ug = ui;  // positions in registers: ui (pgA), ui + 1 (pgB)
  uint4 pgA = load_gm(ug);
  advance(ug);
  uint4 pgB = load_gm(ug);
  advance(ug);
  set_afac(0);

  bool abort = false, fail = false;
  int sq = 0, si = S - 1;  // stage of chunk q, stage of the next chunk to issue
  Cur uq = {0, 0};         // chunk q
  for (int q = 0; q < total; ++q) {
    cp_async_wait<S - 2>();  // this thread's copies of chunk q landed
    __syncthreads();
    form(sq);
    tc::fence_async_smem();
    tc::tc_fence_before();
    abort = __syncthreads_or(fail);
    if (abort) break;
    if (tid == 0) {
      tc::tc_fence_after();
      const uint32_t xh = sbase + (uint32_t)sq * STAGE, xl = xh + X_BYTES;
      const uint32_t yh = xh + 2 * X_BYTES, yl = yh + Y_BYTES;
      const uint32_t d = taddr + (uint32_t)((q & 1) * Cfg::BUF);
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) {
        const uint32_t ko = ks * 32;
        tc::mma_bf16(d, tc::desc_sw128(xh + ko), tc::desc_sw128(yl + ko), idesc, ks > 0 ? 1u : 0u);
        tc::mma_bf16(d, tc::desc_sw128(xl + ko), tc::desc_sw128(yh + ko), idesc, 1u);
      }
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) {
        const uint32_t ko = ks * 32;
        tc::mma_bf16(d, tc::desc_sw128(xh + ko), tc::desc_sw128(yh + ko), idesc, 1u);
      }
      tc::mma_commit(&bar[q & 1]);
    }
    // read back the previous chunk while this one runs, then refill its stage
    if (q >= 1) {
      const int qp = q - 1;
      if (!tc::mbar_wait(&bar[qp & 1], (qp >> 1) & 1, VT_SPINS)) {
        atomicExch(V.status, 1);
        fail = true;
      }
      tc::tc_fence_after();
      consume(qp & 1);
      if (uq.c == 0) {  // qp closed its local-field tile
        write_out(uq.gt - 1);
        set_afac(uq.gt);
      }
    }
    if (!fail) issue(ui, si, pgA);
    else cp_async_commit();
    advance(ui);
    si = si + 1 == S ? 0 : si + 1;
    sq = sq + 1 == S ? 0 : sq + 1;
    advance(uq);
    pgA = pgB;
    pgB = load_gm(ug);
    advance(ug);
  }
  cp_async_wait<0>();
  if (!abort) {
    const int ql = total - 1;
    if (!tc::mbar_wait(&bar[ql & 1], (ql >> 1) & 1, VT_SPINS)) {
      atomicExch(V.status, 1);
      fail = true;
    }
    tc::tc_fence_after();
    consume(ql & 1);
    write_out(ngt - 1);
  }
  abort = __syncthreads_or(fail || abort);
  if (abort && tid == 0) {
    for (int b = 0; b < 2; ++b) tc::mbar_wait(&bar[b], 0, 1024), tc::mbar_wait(&bar[b], 1, 1024);
  }
  // vertex magnitude for the accumulation's operand scaling
  for (int o = 16; o > 0; o >>= 1) amx = fmaxf(amx, __shfl_xor_sync(0xffffffffu, amx, o));
  if (lane == 0) atomicMax(V.amax, __float_as_uint(amx));
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, Cfg::NCOL);
}

// b(i) = Gcar (R1 G1_i)_mu of every FBZ k-point of the launch, pre-scaled by
// sB / 2^14; zero beyond nsum.
__global__ void k_vtx_btab(VtxTcCtx V, int nk, float* __restrict__ out) {
  const size_t n = (size_t)nk * V.nsum_max;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int kl = (int)(e / V.nsum_max), i = (int)(e % V.nsum_max);
    const int* km = V.kmap + 5 * (V.k0 + kl);
    const int K1 = km[0];
    const int nsum = V.legacy ? V.nsum_legacy : V.npw[K1];
    float b = 0.f;
    if (i < nsum) {
      const double* R = V.Rcart + 9 * km[1] + 3 * V.comp;
      const double* g1 = V.G + 3 * V.gidx[(size_t)K1 * V.npwx + i];
      b = (float)(V.Gcar * (R[0] * g1[0] + R[1] * g1[1] + R[2] * g1[2])) * V.sB * (1.0f / 16384.0f);
    }
    out[e] = b;
  }
}

static double pow2_floor_v(double x) { return std::ldexp(1.0, (int)std::floor(std::log2(x))); }

template <int NB, bool CURRENT>
static int launch_vtc(rpa_ctx* c, const VtxTcCtx& V, int nk) {
  using Cfg = VtCfg<NB, CURRENT>;
  auto kern = k_vertex_tc<NB, CURRENT>;
  RPA_CUDA(c, allow_dynamic_smem(kern, c->device));
  kern<<<nk, VT_THREADS, Cfg::SMEM, c->stream>>>(V);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

template <bool CURRENT>
static int launch_vtc_nb(rpa_ctx* c, const VtxTcCtx& V, int nk, int NB) {
  if (NB == 8) return launch_vtc<8, CURRENT>(c, V, nk);
  if (NB == 16) return launch_vtc<16, CURRENT>(c, V, nk);
  return launch_vtc<32, CURRENT>(c, V, nk);
}

// One launch per pair of band windows [m0 + i mwin, ...) x [n0 + j nwin, ...).
template <bool CURRENT>
static int launch_windows(rpa_ctx* c, VtxTcCtx V, int nk, int m0, int mcount, int mwin, int n0, int ncount,
                          int nwin) {
  for (int mb = 0; mb < mcount; mb += mwin) {
    for (int nb = 0; nb < ncount; nb += nwin) {
      V.m0 = m0 + mb;
      V.mcount = std::min(mwin, mcount - mb);
      V.n0 = n0 + nb;
      V.ncount = std::min(nwin, ncount - nb);
      V.gpt = 128 / V.mcount;
      const int NB = V.ncount <= 8 ? 8 : (V.ncount <= 16 ? 16 : 32);
      RPA_TRY(launch_vtc_nb<CURRENT>(c, V, nk, NB));
    }
  }
  return RPA_OK;
}

// Mixed-path vertices of the FBZ k-points [k0, k0+nk) on the tensor cores.
// Leaves *used false when the plane-wave count does not fit the int16 Gfast
// positions (the caller then uses the CUDA-core kernel).
int vertices_tc(rpa_ctx* c, const Chi0Plan& P, int k0, int nk, long long n_trans, const int* pos_of, float2* Mf,
                float2* Mf2, unsigned* amax, bool* used) {
  *used = false;
  if (n_trans == 0) return RPA_OK;
  const bool current = P.mode == RPA_MODE_CURRENT;
  const bool two = current && (P.pol == RPA_POL_YZ || P.pol == RPA_POL_ZY);
  int m0, mcount, n0, ncount;
  if (current) {
    m0 = 0, mcount = c->nbnd, n0 = 0, ncount = c->nbnd;
  } else {
    m0 = P.nocc, mcount = c->nbnd - P.nocc, n0 = 0, ncount = P.nocc;
  }
  if (mcount < 1 || ncount < 1 || c->npwx > 32767) return RPA_OK;
  // band windows of at most 32 on each side, one launch per pair of windows
  // (transitions outside a launch's windows are skipped by it)
  const int nmw = (mcount + 31) / 32, nnw = (ncount + 31) / 32;
  const int mwin = (mcount + nmw - 1) / nmw, nwin = (ncount + nnw - 1) / nnw;
  // Gfast map of the chunk (int16 positions), shared by the chains of one q-point
  int nsum_max = 0;
  for (int i = 0; i < nk; ++i) {
    int K1 = c->h_kmap[5 * (size_t)(k0 + i)];
    nsum_max = std::max(nsum_max, c->legacy ? P.nsum_legacy : c->h_npw[K1]);
  }
  nsum_max = (nsum_max + VT_I - 1) / VT_I * VT_I;
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
  VtxTcCtx V;
  V.kmap = c->d_kmap.as<int>();
  V.ktot = c->d_ktot.as<double>();
  V.G = c->d_G.as<double>();
  V.Rcart = c->d_Rcart.as<double>();
  V.gidx = c->d_gidx.as<int>();
  V.npw = c->d_npw.as<int>();
  V.Glf = c->d_Glf.as<double>();
  V.coeffs = c->d_coeffs.as<uint2>();
  V.gmap = c->d_gmap.as<int16_t>();
  V.btab = nullptr;
  V.trans = c->d_trans.as<Trans>();
  V.offsets = c->d_offsets.as<long long>();
  V.pos_of = pos_of;
  V.status = c->d_flags.as<int>() + 3;
  V.k0 = k0;
  V.nlf = c->nlf;
  V.npwx = c->npwx;
  V.nbnd = c->nbnd;
  V.legacy = c->legacy ? 1 : 0;
  V.nsum_legacy = P.nsum_legacy;
  V.nsum_max = nsum_max;
  V.q0 = c->q[0];
  V.q1 = c->q[1];
  V.q2 = c->q[2];
  V.Gcar = P.Gcar;
  if (!current) {
    V.comp = 0;
    V.sB = 1.0f;
    V.a_scale = 0.0f;
    V.out_scale = (float)(1.0 / (16384.0 * 16384.0));
    V.M = Mf;
    V.amax = amax;
    *used = true;
    return launch_windows<false>(c, V, nk, m0, mcount, mwin, n0, ncount, nwin);
  }
  // current vertices: |C| <= 1 (orthonormal bands), |b(i)| <= Gcar max|G|
  double gmax = 0.0;
  for (size_t g = 0; g < c->h_G.size() / 3; ++g) {
    const double* v = &c->h_G[3 * g];
    gmax = std::max(gmax, std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
  }
  const double bmax = std::max(P.Gcar * gmax, 1e-30);
  V.sB = (float)(16384.0 / pow2_floor_v(bmax * 1.5));
  V.a_scale = V.sB / 16384.0f;
  V.out_scale = (float)(1.0 / (16384.0 * (double)V.sB));
  int comps[2];
  switch (P.pol) {
    case RPA_POL_XX: comps[0] = comps[1] = 0; break;
    case RPA_POL_YY: comps[0] = comps[1] = 1; break;
    case RPA_POL_ZZ: comps[0] = comps[1] = 2; break;
    case RPA_POL_YZ: comps[0] = 1; comps[1] = 2; break;
    default: comps[0] = 2; comps[1] = 1; break;
  }
  RPA_TRY(ensure(c, c->d_vbt, sizeof(float) * (size_t)nk * nsum_max));
  V.btab = c->d_vbt.as<float>();
  // the yz / zy pair: one pass per Cartesian component
  for (int a = 0; a < (two ? 2 : 1); ++a) {
    V.comp = comps[a];
    V.M = a == 0 ? Mf : Mf2;
    V.amax = amax + a;
    k_vtx_btab<<<2048, 256, 0, c->stream>>>(V, nk, c->d_vbt.as<float>());
    RPA_CUDA(c, cudaGetLastError());
    ++c->launches;
    RPA_TRY(launch_windows<true>(c, V, nk, m0, mcount, mwin, n0, ncount, nwin));
  }
  *used = true;
  return RPA_OK;
}

}  // namespace rpa
