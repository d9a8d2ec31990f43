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
};

constexpr int TC_TT = 32;       // transitions per chunk (K = 64 16-bit values)
constexpr int TC_GA = 128;      // G rows per tile (MMA M)
constexpr int TC_GB = 96;       // G' rows per tile
constexpr int TC_FLUSH = 16;    // chunks summed in FP32 before a double-float flush
constexpr uint32_t TC_SPINS = 1u << 22;

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

template <int NIO, bool CPLX, bool F16>
__global__ void __launch_bounds__(256, 1) k_accum_tc(AccTcCtx A) {
  constexpr int NB = CPLX ? 2 * TC_GB : TC_GB;               // MMA N
  constexpr int DCOLS = NIO * NB;                            // TMEM columns per buffer
  static_assert(DCOLS == 192, "one warpgroup column half = 96 columns");
  constexpr uint32_t A_BYTES = TC_GA * 128, B_BYTES = NB * 128;
  constexpr uint32_t STAGE = 2 * B_BYTES + NIO * 2 * A_BYTES;  // Bh, Bl, (Ah, Al) x NIO
  constexpr uint32_t NCOL = 512;                               // 2 x 192 used

  extern __shared__ unsigned char smraw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tslot;
  __shared__ float wtab[2][NIO][TC_TT];
  __shared__ int range[2];

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r0 = blockIdx.x * NIO;
  const int g0 = blockIdx.y * TC_GA, h0 = blockIdx.z * TC_GB;
  const int nrowA = min(TC_GA, A.nlf - g0), nrowB = min(TC_GB, A.nlf - h0);
  const size_t np = (size_t)A.nlf * A.nlf;

  auto Bh = [&](int s) { return base + s * STAGE; };
  auto Bl = [&](int s) { return base + s * STAGE + B_BYTES; };
  auto Ah = [&](int s, int j) { return base + s * STAGE + 2 * B_BYTES + j * 2 * A_BYTES; };
  auto Al = [&](int s, int j) { return base + s * STAGE + 2 * B_BYTES + j * 2 * A_BYTES + A_BYTES; };

  if (warp == 0) {
    tc::tmem_alloc(&tslot, NCOL);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    tc::fence_mbar_init();
    range[0] = lb_lo(A.rec, A.n_inter, r0 - A.wmax + 1);
    range[1] = lb_lo(A.rec, A.n_inter, r0 + NIO);
  }
  // zero both stages once: padding rows stay zero for the whole kernel
  for (uint32_t e = tid; e < 2 * STAGE / 16; e += 256) reinterpret_cast<uint4*>(base)[e] = make_uint4(0, 0, 0, 0);
  tc::fence_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t taddr = tslot;
  const int ta = range[0], tb = range[1];
  const int nchunks = (tb - ta + TC_TT - 1) / TC_TT;
  const uint32_t idesc = tc::idesc_bf16(TC_GA, NB, F16);

  // this thread's slice of the accumulator: TMEM lane quarter wq, column half hf
  const int wq = warp & 3, hf = warp >> 2;
  const int grow = g0 + wq * 32 + lane;               // G
  const int io_t = CPLX ? r0 : r0 + hf;                // frequency row of this slice
  const int comp = CPLX ? hf : 0;                       // Re / Im
  float acc[96];
#pragma unroll
  for (int i = 0; i < 96; ++i) acc[i] = 0.f;

  auto consume = [&](int buf) {
#pragma unroll
    for (int c0 = 0; c0 < 96; c0 += 32) {
      float v[32];
      tc::tmem_ld32(taddr + ((uint32_t)(wq * 32) << 16) + (uint32_t)(buf * DCOLS + hf * 96 + c0), v);
      tc::tmem_ld_wait();
#pragma unroll
      for (int i = 0; i < 32; ++i) acc[c0 + i] += v[i];
    }
  };
  auto flush = [&]() {
    if (grow < A.nlf && io_t < A.nw) {
      const int ncomp = CPLX ? 2 : 1;
#pragma unroll 4
      for (int j = 0; j < 96; ++j) {
        if (j < nrowB) {
          size_t p = (size_t)grow + (size_t)A.nlf * (h0 + j);
          float2* dst = A.Sdf + ((size_t)io_t * np + p) * ncomp + comp;
          *dst = df_add(*dst, acc[j] * A.inv_scale);
        }
        acc[j] = 0.f;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 96; ++j) acc[j] = 0.f;
    }
  };

  bool abort = false;
  int last_commit = -1, consumed = 0;

  for (int c = 0; c < nchunks && !abort; ++c) {
    const int s = c & 1;
    const int ts = ta + c * TC_TT;
    if (c >= 2) {
      bool ok = tc::mbar_wait(&bar[s], ((c - 2) >> 1) & 1, TC_SPINS);
      if (!ok) atomicExch(A.status, 1);
      abort = __syncthreads_or(!ok);
      if (abort) break;
      tc::tc_fence_after();
      consume(s);  // result of chunk c-2
      tc::tc_fence_before();
      if (++consumed % TC_FLUSH == 0) flush();
    }
    // Lorentzian weights of this chunk for the NIO rows (scaled)
    if (tid < NIO * TC_TT) {
      int j = tid / TC_TT, tt = tid % TC_TT, t = ts + tt, r = r0 + j;
      float w = 0.f;
      if (t < tb && r < A.nw) {
        const Trans& R = A.rec[t];
        if (r >= R.lo && r <= R.hi) {
          bool in;
          double L = lorentz_tc(A, r, R.e1, R.e2, &in);
          if (in) w = (float)(R.c * L * A.scaleA);
        }
      }
      wtab[s][j][tt] = w;
    }
    __syncthreads();
    // A tiles: rows G = g0 + row, 8 transitions per task
    for (int e = tid; e < nrowA * 4; e += 256) {
      const int row = e % nrowA, grp = e / nrowA;
      float re[8], im[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        int t = ts + grp * 8 + q;
        float2 m = t < A.n_inter ? A.M[(size_t)t * A.nlf + g0 + row] : make_float2(0.f, 0.f);
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
    // B tiles: rows G' = h0 + row (and 96 + row for the imaginary part)
    for (int e = tid; e < nrowB * 4; e += 256) {
      const int row = e % nrowB, grp = e / nrowB;
      float re[8], im[8], nim[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        int t = ts + grp * 8 + q;
        float2 m = t < A.n_inter ? A.M2[(size_t)t * A.nlf + h0 + row] : make_float2(0.f, 0.f);
        re[q] = m.x * A.scaleB;
        im[q] = m.y * A.scaleB;
        nim[q] = -im[q];
      }
      uint4 hi, lo;
      split8<F16>(re, hi, lo);
      st16(Bh(s), row, grp, hi);
      st16(Bl(s), row, grp, lo);
      if (CPLX) {
        st16(Bh(s), TC_GB + row, 4 + grp, hi);
        st16(Bl(s), TC_GB + row, 4 + grp, lo);
      }
      split8<F16>(im, hi, lo);
      st16(Bh(s), row, 4 + grp, hi);
      st16(Bl(s), row, 4 + grp, lo);
      if (CPLX) {
        split8<F16>(nim, hi, lo);
        st16(Bh(s), TC_GB + row, grp, hi);
        st16(Bl(s), TC_GB + row, grp, lo);
      }
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::tc_fence_after();
      const uint32_t bh = tc::smem_u32(Bh(s)), bl = tc::smem_u32(Bl(s));
#pragma unroll
      for (int j = 0; j < NIO; ++j) {
        const uint32_t ah = tc::smem_u32(Ah(s, j)), al = tc::smem_u32(Al(s, j));
        const uint32_t d = taddr + (uint32_t)(s * DCOLS + j * NB);
        // cross products first (fresh accumulator), the large hi*hi products last
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          const uint32_t ko = ks * 32;
          tc::mma_bf16(d, tc::desc_sw128(ah + ko), tc::desc_sw128(bl + ko), idesc, ks > 0 ? 1u : 0u);
          tc::mma_bf16(d, tc::desc_sw128(al + ko), tc::desc_sw128(bh + ko), idesc, 1u);
        }
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          const uint32_t ko = ks * 32;
          tc::mma_bf16(d, tc::desc_sw128(ah + ko), tc::desc_sw128(bh + ko), idesc, 1u);
        }
      }
      tc::mma_commit(&bar[s]);
    }
    last_commit = c;
  }
  // drain the last (up to) two chunks
  if (!abort) {
    for (int cc = (nchunks >= 2 ? nchunks - 2 : 0); cc < nchunks; ++cc) {
      const int s = cc & 1;
      bool ok = tc::mbar_wait(&bar[s], (cc >> 1) & 1, TC_SPINS);
      if (!ok) atomicExch(A.status, 1);
      abort = __syncthreads_or(!ok);
      if (abort) break;
      tc::tc_fence_after();
      consume(s);
      tc::tc_fence_before();
    }
    if (!abort) flush();
  }
  if (abort && tid == 0 && last_commit >= 0) {
    // let the MMAs already issued finish before the TMEM is released
    tc::mbar_wait(&bar[last_commit & 1], (last_commit >> 1) & 1, TC_SPINS);
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}

// Sorted FP32 copies of the FP64 vertices, Mf[i] = M[order[i]], and the
// largest |component| (as float bits) for the power-of-two operand scaling.
__global__ void k_pack_sorted(const Trans* __restrict__ rec, const double2* __restrict__ M, float2* __restrict__ Mf,
                              int n, int nlf, unsigned* amax) {
  size_t tot = (size_t)n * nlf;
  float mx = 0.f;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    size_t i = e / nlf;
    int g = (int)(e % nlf);
    double2 v = M[(size_t)rec[i].k * nlf + g];
    float2 f = make_float2((float)v.x, (float)v.y);
    Mf[e] = f;
    mx = fmaxf(mx, fmaxf(fabsf(f.x), fabsf(f.y)));
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(amax, __float_as_uint(mx));
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

template <int NIO, bool CPLX, bool F16>
static int launch_tc(rpa_ctx* c, const AccTcCtx& A, int nw) {
  constexpr int NB = CPLX ? 2 * TC_GB : TC_GB;
  constexpr size_t STAGE = 2 * (size_t)NB * 128 + (size_t)NIO * 2 * TC_GA * 128;
  const size_t smem = 2 * STAGE + 1024;
  auto kern = k_accum_tc<NIO, CPLX, F16>;
  RPA_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((nw + NIO - 1) / NIO, (A.nlf + TC_GA - 1) / TC_GA, (A.nlf + TC_GB - 1) / TC_GB);
  kern<<<grid, 256, smem, c->stream>>>(A);
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
  if (P.mode == RPA_MODE_CURRENT)
    return f16 ? launch_tc<1, true, true>(c, A, P.nw) : launch_tc<1, true, false>(c, A, P.nw);
  return f16 ? launch_tc<2, false, true>(c, A, P.nw) : launch_tc<2, false, false>(c, A, P.nw);
}

// Packs the sorted FP32 vertices and returns the scaling statistics.
int pack_sorted_fp32(rpa_ctx* c, int n_inter, float2* Mf, float2* Mf2, bool two, float* amaxM, float* amaxM2,
                     double* cmax) {
  *amaxM = *amaxM2 = 0.f;
  *cmax = 0.0;
  if (n_inter == 0) return RPA_OK;
  RPA_TRY(ensure(c, c->d_ntrans, 32));
  RPA_CUDA(c, cudaMemsetAsync(c->d_ntrans.p, 0, 32, c->stream));
  unsigned* am = c->d_ntrans.as<unsigned>();
  k_pack_sorted<<<2048, 256, 0, c->stream>>>(c->d_sorted.as<Trans>(), c->d_M.as<double2>(), Mf, n_inter, c->nlf, am);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  if (two) {
    k_pack_sorted<<<2048, 256, 0, c->stream>>>(c->d_sorted.as<Trans>(), c->d_M2.as<double2>(), Mf2, n_inter,
                                               c->nlf, am + 1);
    RPA_CUDA(c, cudaGetLastError());
    ++c->launches;
  }
  k_cmax<<<256, 256, 0, c->stream>>>(c->d_sorted.as<Trans>(), n_inter,
                                     reinterpret_cast<unsigned long long*>(c->d_ntrans.as<char>() + 8));
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  unsigned char h[16];
  RPA_CUDA(c, cudaMemcpyAsync(h, c->d_ntrans.p, 16, cudaMemcpyDeviceToHost, c->stream));
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  unsigned u0, u1;
  std::memcpy(&u0, h, 4);
  std::memcpy(&u1, h + 4, 4);
  std::memcpy(cmax, h + 8, 8);
  std::memcpy(amaxM, &u0, 4);
  std::memcpy(amaxM2, &u1, 4);
  if (!two) *amaxM2 = *amaxM;
  return RPA_OK;
}

int df_to_f64(rpa_ctx* c, size_t n) {
  k_df_to_f64<<<2048, 256, 0, c->stream>>>(c->d_Sdf.as<float2>(), c->d_S.as<double>(), n);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

}  // namespace rpa
