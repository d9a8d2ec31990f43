// k_vertex_tc.cu -- plane-wave vertices on the tcgen05 tensor cores (mixed path).
//
// Same vertices as k_vertex.cu (genMnmK1K2, Sloss.f90:883-952; genStrujniVrhovi,
// Optabs.f90:1354-1472), written per FBZ k-point as a GEMM over the plane
// waves i of K1:
//     M_nm(G) = sum_i conj(C1[n,i]) * f(G,i) * C2[m, Gfast(G,i)]
// rows = (G, m) pairs (4 local fields x 32 bands of K2 per 128-row tile),
// columns = bands n of K1, K = plane waves.  Complex values are folded into
// one real GEMM by stacking the K axis (32 plane waves -> 64 K columns):
//     X((G,m), :) = [ Re y | Im y ],   y = f(G,i) C2[m, Gfast(G,i)]
//     Y(n, :)     = [ Re c | Im c ]  ->  D((G,m), n)        = Re M
//     Y(NB+n, :)  = [ -Im c | Re c ] ->  D((G,m), NB + n)   = Im M      (c = C1[n,i])
// The current factor of Optabs separates, f(G,i) = 0.5 Gcar (q + 2k + Glf_G)_mu
// + Gcar (R1 G1_i)_mu, so it costs one add per element.  Operands are split
// into power-of-two-scaled fp16 hi + lo halves (D = Xh Yh + Xh Yl + Xl Yh); each
// 32-plane-wave chunk accumulates in a fresh TMEM buffer (two, ping-pong) that
// is added to FP32 registers, as in k_accum_tc.cu.  The Gfast map comes
// precomputed (k_gmap) as int16 basis positions.  Results go straight to the
// window-sorted vertex rows pos_of[t] read by the accumulation.

#include <cuda_fp16.h>

#include <cmath>

#include "rpa_internal.cuh"
#include "tc05.cuh"

namespace rpa {

struct MapCtx;  // k_vertex.cu
int build_gmap(rpa_ctx* c, int k0, int nk, int nsum_max, int16_t* gmap, int nsum_legacy);

struct VtxTcCtx {
  const int* kmap;
  const double* ktot;
  const double* G;        // Cartesian G list
  const double* Rcart;    // [48][9]
  const int* gidx;        // [kibz][npwx]
  const int* npw;
  const double* Glf;      // [nlf][3]
  const float2* coeff;    // FP32 coefficients [kibz][npwx][nbnd]
  const int16_t* gmap;    // [k_local][nlf][nsum_max]
  const Trans* trans;
  const long long* offsets;
  const int* pos_of;
  float2* M;
  float2* M2;
  unsigned* amax;
  int* status;
  int k0, nlf, npwx, nbnd, legacy, nsum_legacy, nsum_max;
  int m0, mcount, n0, ncount;
  int ca, cb;
  double q0, q1, q2, Gcar;
  float sX, sY, inv_scale;
};

constexpr int VT_I = 32;      // plane waves per chunk (K = 64)
constexpr int VT_MB = 32;     // K2 bands per local field in a tile
constexpr int VT_GPT = 4;     // local fields per 128-row tile
constexpr uint32_t VT_SPINS = 1u << 22;

__device__ __forceinline__ void st16v(unsigned char* tile, int row, int chunk, uint4 v) {
  *reinterpret_cast<uint4*>(tile + row * 128 + ((chunk ^ (row & 7)) << 4)) = v;
}

__device__ __forceinline__ void split8h(const float* x, uint4& hi, uint4& lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    __half2 hh = __floats2half2_rn(x[2 * i], x[2 * i + 1]);
    float2 f = __half22float2(hh);
    __half2 ll = __floats2half2_rn(x[2 * i] - f.x, x[2 * i + 1] - f.y);
    h[i] = *reinterpret_cast<uint32_t*>(&hh);
    l[i] = *reinterpret_cast<uint32_t*>(&ll);
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// NB: bands n per tile (8, 16 or 32); N = 2 NB.  NACC = 2 for the yz/zy pair.
template <int NB, bool CURRENT, bool TWO>
__global__ void __launch_bounds__(256, 2) k_vertex_tc(VtxTcCtx V) {
  constexpr int N = 2 * NB;
  constexpr int NACC = TWO ? 2 : 1;
  constexpr uint32_t X_BYTES = 128 * 128, Y_BYTES = N * 128;
  constexpr uint32_t STAGE = NACC * 2 * X_BYTES + 2 * Y_BYTES;  // (Xh, Xl) x NACC, Yh, Yl
  constexpr int DCOLS = NACC * N;                               // TMEM columns per buffer
  constexpr uint32_t NCOL = 2 * DCOLS <= 32 ? 32 : 2 * DCOLS <= 64 ? 64 : 2 * DCOLS <= 128 ? 128 : 256;

  extern __shared__ unsigned char smraw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tslot;
  __shared__ int ptab[32][VT_MB];            // sorted vertex row of (n - n0, m - m0), -1 if none
  __shared__ float bfac[2][VT_I][2];         // b(i) for the two current components
  __shared__ float afac[VT_GPT][2];          // a(G)

  auto Xh = [&](int s, int a) { return base + s * STAGE + a * 2 * X_BYTES; };
  auto Xl = [&](int s, int a) { return base + s * STAGE + a * 2 * X_BYTES + X_BYTES; };
  auto Yh = [&](int s) { return base + s * STAGE + NACC * 2 * X_BYTES; };
  auto Yl = [&](int s) { return base + s * STAGE + NACC * 2 * X_BYTES + Y_BYTES; };

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int kl = blockIdx.x, ik = V.k0 + kl;
  const long long t0 = V.offsets[kl], t1 = V.offsets[kl + 1];
  if (t1 == t0) return;
  const int* km = V.kmap + 5 * ik;
  const int K1 = km[0], R1 = km[1], K2 = km[2];
  const int nsum = V.legacy ? V.nsum_legacy : V.npw[K1];
  const int nchunk = (nsum + VT_I - 1) / VT_I;
  const int ngt = (V.nlf + VT_GPT - 1) / VT_GPT;
  const int total = ngt * nchunk;

  if (warp == 0) {
    tc::tmem_alloc(&tslot, NCOL);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    tc::fence_mbar_init();
  }
  for (int e = tid; e < 32 * VT_MB; e += 256) (&ptab[0][0])[e] = -1;
  for (uint32_t e = tid; e < 2 * STAGE / 16; e += 256) reinterpret_cast<uint4*>(base)[e] = make_uint4(0, 0, 0, 0);
  tc::fence_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  for (long long t = t0 + tid; t < t1; t += 256) {
    int nm = V.trans[t].nm;
    int n = (nm & 0xffff) - V.n0, m = (nm >> 16) - V.m0;
    if (n >= 0 && n < V.ncount && m >= 0 && m < V.mcount) ptab[n][m] = V.pos_of[t];
  }
  const uint32_t taddr = tslot;
  const uint32_t idesc = tc::idesc_bf16(128, N, true);
  const double* kv = V.ktot + 3 * ik;
  const float2* C1 = V.coeff + (size_t)K1 * V.npwx * V.nbnd;
  const float2* C2 = V.coeff + (size_t)K2 * V.npwx * V.nbnd;
  const int16_t* gm = V.gmap + (size_t)kl * V.nlf * V.nsum_max;

  // accumulator slice of this thread: row = TMEM lane, columns half hf
  const int wq = warp & 3, hf = warp >> 2;
  const int row_t = wq * 32 + lane;  // (G_local = wq, m = lane)
  float acc[NACC][NB];
#pragma unroll
  for (int a = 0; a < NACC; ++a)
#pragma unroll
    for (int j = 0; j < NB; ++j) acc[a][j] = 0.f;

  auto consume = [&](int buf) {
#pragma unroll
    for (int a = 0; a < NACC; ++a) {
      const uint32_t ad = taddr + ((uint32_t)(wq * 32) << 16) + (uint32_t)(buf * DCOLS + a * N + hf * NB);
      float v[NB];
      if (NB == 32) tc::tmem_ld32(ad, v);
      else if (NB == 16) tc::tmem_ld16(ad, v);
      else tc::tmem_ld8(ad, v);
      tc::tmem_ld_wait();
#pragma unroll
      for (int j = 0; j < NB; ++j) acc[a][j] += v[j];
    }
  };
  float amx[NACC];
#pragma unroll
  for (int a = 0; a < NACC; ++a) amx[a] = 0.f;
  auto write_out = [&](int gt) {
    const int G = gt * VT_GPT + wq;
    const int m = lane;
    if (G < V.nlf && m < V.mcount) {
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        int r = j < V.ncount ? ptab[j][m] : -1;
        if (r >= 0) {
#pragma unroll
          for (int a = 0; a < NACC; ++a) {
            float v = acc[a][j] * V.inv_scale;
            float* dst = reinterpret_cast<float*>((a == 0 ? V.M : V.M2) + (size_t)r * V.nlf + G) + hf;
            *dst = v;
            amx[a] = fmaxf(amx[a], fabsf(v));
          }
        }
      }
    }
#pragma unroll
    for (int a = 0; a < NACC; ++a)
#pragma unroll
      for (int j = 0; j < NB; ++j) acc[a][j] = 0.f;
  };

  bool abort = false;
  for (int q = 0; q < total && !abort; ++q) {
    const int s = q & 1;
    const int gt = q / nchunk, c = q % nchunk, i0 = c * VT_I;
    // per-chunk factors: b(i) (current vertices) and a(G)
    if (CURRENT) {
      if (tid < VT_I) {
        int i = i0 + tid;
        float b0 = 0.f, b1 = 0.f;
        if (i < nsum) {
          const double* g1 = V.G + 3 * V.gidx[(size_t)K1 * V.npwx + i];
          const double* R = V.Rcart + 9 * R1;
          double k3[3] = {R[0] * g1[0] + R[1] * g1[1] + R[2] * g1[2], R[3] * g1[0] + R[4] * g1[1] + R[5] * g1[2],
                          R[6] * g1[0] + R[7] * g1[1] + R[8] * g1[2]};
          b0 = (float)(V.Gcar * k3[V.ca]);
          b1 = (float)(V.Gcar * k3[V.cb]);
        }
        bfac[s][tid][0] = b0;
        bfac[s][tid][1] = b1;
      } else if (tid < VT_I + VT_GPT && c == 0) {
        int G = gt * VT_GPT + (tid - VT_I);
        float a0 = 0.f, a1 = 0.f;
        if (G < V.nlf) {
          const double* gl = V.Glf + 3 * G;
          double j3[3] = {V.q0 + 2.0 * kv[0] + gl[0], V.q1 + 2.0 * kv[1] + gl[1], V.q2 + 2.0 * kv[2] + gl[2]};
          a0 = (float)(0.5 * V.Gcar * j3[V.ca]);
          a1 = (float)(0.5 * V.Gcar * j3[V.cb]);
        }
        afac[tid - VT_I][0] = a0;
        afac[tid - VT_I][1] = a1;
      }
      __syncthreads();
    }
    // X tiles: row = (G_local, m), 8 plane waves per task
    for (int e = tid; e < 128 * 4; e += 256) {
      const int row = e & 127, grp = e >> 7;
      const int gl = row >> 5, m = row & 31, G = gt * VT_GPT + gl;
      float xr[NACC][8], xi[NACC][8];
      if (G < V.nlf && m < V.mcount) {
        const int ib = i0 + grp * 8;
        int16_t pos[8];
        *reinterpret_cast<uint4*>(pos) = *reinterpret_cast<const uint4*>(gm + (size_t)G * V.nsum_max + ib);
#pragma unroll
        for (int qq = 0; qq < 8; ++qq) {
          float2 v = make_float2(0.f, 0.f);
          if (ib + qq < nsum && pos[qq] >= 0) v = C2[(size_t)pos[qq] * V.nbnd + V.m0 + m];
          if (CURRENT) {
            float f0 = (afac[gl][0] + bfac[s][grp * 8 + qq][0]) * V.sX;
            xr[0][qq] = v.x * f0;
            xi[0][qq] = v.y * f0;
            if (TWO) {
              float f1 = (afac[gl][1] + bfac[s][grp * 8 + qq][1]) * V.sX;
              xr[NACC - 1][qq] = v.x * f1;
              xi[NACC - 1][qq] = v.y * f1;
            }
          } else {
            xr[0][qq] = v.x * V.sX;
            xi[0][qq] = v.y * V.sX;
          }
        }
      } else {
#pragma unroll
        for (int a = 0; a < NACC; ++a)
#pragma unroll
          for (int qq = 0; qq < 8; ++qq) xr[a][qq] = xi[a][qq] = 0.f;
      }
#pragma unroll
      for (int a = 0; a < NACC; ++a) {
        uint4 hi, lo;
        split8h(xr[a], hi, lo);
        st16v(Xh(s, a), row, grp, hi);
        st16v(Xl(s, a), row, grp, lo);
        split8h(xi[a], hi, lo);
        st16v(Xh(s, a), row, 4 + grp, hi);
        st16v(Xl(s, a), row, 4 + grp, lo);
      }
    }
    // Y tiles: rows n (Re part) and NB + n (Im part)
    for (int e = tid; e < NB * 4; e += 256) {
      const int n = e % NB, grp = e / NB;
      float cr[8], ci[8], nci[8];
#pragma unroll
      for (int qq = 0; qq < 8; ++qq) {
        int i = i0 + grp * 8 + qq;
        float2 v = (n < V.ncount && i < nsum) ? C1[(size_t)i * V.nbnd + V.n0 + n] : make_float2(0.f, 0.f);
        cr[qq] = v.x * V.sY;
        ci[qq] = v.y * V.sY;
        nci[qq] = -ci[qq];
      }
      uint4 hi, lo;
      split8h(cr, hi, lo);
      st16v(Yh(s), n, grp, hi);
      st16v(Yl(s), n, grp, lo);
      st16v(Yh(s), NB + n, 4 + grp, hi);
      st16v(Yl(s), NB + n, 4 + grp, lo);
      split8h(ci, hi, lo);
      st16v(Yh(s), n, 4 + grp, hi);
      st16v(Yl(s), n, 4 + grp, lo);
      split8h(nci, hi, lo);
      st16v(Yh(s), NB + n, grp, hi);
      st16v(Yl(s), NB + n, grp, lo);
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::tc_fence_after();
      const uint32_t yh = tc::smem_u32(Yh(s)), yl = tc::smem_u32(Yl(s));
#pragma unroll
      for (int a = 0; a < NACC; ++a) {
        const uint32_t xh = tc::smem_u32(Xh(s, a)), xl = tc::smem_u32(Xl(s, a));
        const uint32_t d = taddr + (uint32_t)(s * DCOLS + a * N);
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
      }
      tc::mma_commit(&bar[s]);
    }
    // read back the previous chunk while this one runs
    if (q >= 1) {
      const int qp = q - 1;
      bool ok = tc::mbar_wait(&bar[s ^ 1], (qp >> 1) & 1, VT_SPINS);
      if (!ok) atomicExch(V.status, 1);
      abort = __syncthreads_or(!ok);
      if (abort) break;
      tc::tc_fence_after();
      consume(s ^ 1);
      tc::tc_fence_before();
      if (qp % nchunk == nchunk - 1) write_out(qp / nchunk);
    }
    __syncthreads();
  }
  if (!abort && total > 0) {
    const int ql = total - 1;
    bool ok = tc::mbar_wait(&bar[ql & 1], (ql >> 1) & 1, VT_SPINS);
    if (!ok) atomicExch(V.status, 1);
    abort = __syncthreads_or(!ok);
    if (!abort) {
      tc::tc_fence_after();
      consume(ql & 1);
      tc::tc_fence_before();
      write_out(ql / nchunk);
    }
  } else if (abort && tid == 0 && total > 0) {
    for (int b = 0; b < 2; ++b) tc::mbar_wait(&bar[b], 0, 1024), tc::mbar_wait(&bar[b], 1, 1024);
  }
  // vertex magnitude for the accumulation's operand scaling
#pragma unroll
  for (int a = 0; a < NACC; ++a) {
    float mx = amx[a];
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) atomicMax(V.amax + a, __float_as_uint(mx));
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}

static double pow2_floor_v(double x) { return std::ldexp(1.0, (int)std::floor(std::log2(x))); }

template <int NB, bool CURRENT, bool TWO>
static int launch_vtc(rpa_ctx* c, const VtxTcCtx& V, int nk) {
  constexpr int NACC = TWO ? 2 : 1;
  constexpr size_t STAGE = (size_t)NACC * 2 * 128 * 128 + 2 * (size_t)(2 * NB) * 128;
  const size_t smem = 2 * STAGE + 1024;
  auto kern = k_vertex_tc<NB, CURRENT, TWO>;
  RPA_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<nk, 256, smem, c->stream>>>(V);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

// Mixed-path vertices of the FBZ k-points [k0, k0+nk) on the tensor cores.
// Returns RPA_EINVAL when the band windows do not fit one tile (the caller
// then uses the CUDA-core kernel).
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
  if (mcount > VT_MB || ncount > 32 || c->npwx > 32767) return RPA_OK;
  int NB = ncount <= 8 ? 8 : (ncount <= 16 ? 16 : 32);
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
  V.coeff = c->d_coeff32.as<float2>();
  V.gmap = c->d_gmap.as<int16_t>();
  V.trans = c->d_trans.as<Trans>();
  V.offsets = c->d_offsets.as<long long>();
  V.pos_of = pos_of;
  V.M = Mf;
  V.M2 = Mf2;
  V.amax = amax;
  V.status = c->d_flags.as<int>() + 3;
  V.k0 = k0;
  V.nlf = c->nlf;
  V.npwx = c->npwx;
  V.nbnd = c->nbnd;
  V.legacy = c->legacy ? 1 : 0;
  V.nsum_legacy = P.nsum_legacy;
  V.nsum_max = nsum_max;
  V.m0 = m0, V.mcount = mcount, V.n0 = n0, V.ncount = ncount;
  int ca = 0, cb = 0;
  switch (P.pol) {
    case RPA_POL_XX: ca = cb = 0; break;
    case RPA_POL_YY: ca = cb = 1; break;
    case RPA_POL_ZZ: ca = cb = 2; break;
    case RPA_POL_YZ: ca = 1; cb = 2; break;
    default: ca = 2; cb = 1; break;
  }
  V.ca = ca;
  V.cb = cb;
  V.q0 = c->q[0];
  V.q1 = c->q[1];
  V.q2 = c->q[2];
  V.Gcar = P.Gcar;
  // operand scaling: |C| <= 1 (orthonormal bands); |f| bounded by the G vectors in play
  double fmax = 1.0;
  if (current) {
    double gmax = 0.0;
    for (size_t g = 0; g < c->h_G.size() / 3; ++g) {
      const double* v = &c->h_G[3 * g];
      gmax = std::max(gmax, std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
    }
    double kq = 0.0;
    for (int i = 0; i < c->ntot; ++i) {
      const double* k = &c->h_ktot[3 * (size_t)i];
      kq = std::max(kq, std::sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]));
    }
    double qn = std::sqrt(c->q[0] * c->q[0] + c->q[1] * c->q[1] + c->q[2] * c->q[2]);
    fmax = P.Gcar * (0.5 * (qn + 2.0 * kq + gmax) + gmax);
  }
  V.sX = (float)(16384.0 / pow2_floor_v(fmax * 1.5));
  V.sY = 16384.0f;
  V.inv_scale = (float)(1.0 / ((double)V.sX * (double)V.sY));
  *used = true;
  if (!current) {
    if (NB == 8) return launch_vtc<8, false, false>(c, V, nk);
    if (NB == 16) return launch_vtc<16, false, false>(c, V, nk);
    return launch_vtc<32, false, false>(c, V, nk);
  }
  if (two) {
    if (NB == 8) return launch_vtc<8, true, true>(c, V, nk);
    if (NB == 16) return launch_vtc<16, true, true>(c, V, nk);
    return launch_vtc<32, true, true>(c, V, nk);
  }
  if (NB == 8) return launch_vtc<8, true, false>(c, V, nk);
  if (NB == 16) return launch_vtc<16, true, false>(c, V, nk);
  return launch_vtc<32, true, false>(c, V, nk);
}

}  // namespace rpa
