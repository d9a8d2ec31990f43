// k_vertex.cu -- plane-wave vertices M_nm(G) by an integer Miller-index gather.
//
// Reference: genMnmK1K2 (W/Sloss.f90:883-952), genStrujniVrhovi
// (Chi_RPA/Optabs.f90:1354-1472) and their igk-aware forms
// (Modules/vertices.f90:88-189, 293-394).  The reference finds, for every
// local field G and coefficient G1 of K1, the coefficient of K2 at
//     G'' = RI_R2 (R_R1 G1 + Glf_G + G_iG0)
// by a float-eps linear search over the K2 basis (Gfast).  Here the same
// vector is formed in integer crystal coordinates and looked up through a
// dense Miller box table (Miller triple -> G-list index) and, with an igk
// map, the inverse igk table of K2 (G-list index -> basis position).  Both
// give the first (and only) matching position, or "absent" (the reference's
// NG2+1 sentinel), so the map is identical to the reference's.
//
// One block handles one FBZ k-point and a chunk of GC local fields; the
// transitions of that k-point are the rows emitted by k_setup.cu.  Per slice
// of IC coefficients the block stages conj-free C1 rows of K1 and the
// gathered C2 rows of K2 (band-contiguous, so each gather is one coalesced
// row of nbnd complex values), then every thread accumulates its
// (transition, G) outputs in FP64.

#include <climits>

#include "rpa_internal.cuh"

namespace rpa {

struct MapCtx {
  const int* kmap;       // 5 per FBZ k
  const double* ktot;    // 3 per FBZ k
  const int* miller;     // 3 per G
  const double* G;       // 3 per G (Cartesian, 2pi/a0)
  const int* box;        // Miller box -> G index (-1 absent)
  int box_lo0, box_lo1, box_lo2, box_d0, box_d1, box_d2;
  const int* Rc;         // [48][9] row-major integer crystal matrices
  const int* RIc;
  const double* Rcart;   // [48][9] row-major Cartesian R
  const int* npw;        // per IBZ k
  const int* gidx;       // [kibz][npwx] G index of basis position (legacy: identity)
  const int* inv;        // [kibz][ng] basis position of G index (-1 absent); NULL in legacy mode
  int npwx, ng, legacy, nsum_legacy;
  const int* lf_miller;  // 3 per local field
  const double* Glf;     // 3 per local field
  int nlf;
  double q0, q1, q2, Gcar;
};

// Basis position in K2 of G'' for (local field g, coefficient i of K1), or -1.
__device__ __forceinline__ int gfast_pos(const MapCtx& C, const int* km, int g, int i) {
  int K1 = km[0], R1 = km[1], K2 = km[2], R2 = km[3], iG0 = km[4];
  int gi = C.gidx[(size_t)K1 * C.npwx + i];
  const int* m1 = C.miller + 3 * gi;
  int a0 = m1[0], a1 = m1[1], a2 = m1[2];
  const int* r = C.Rc + 9 * R1;
  int b0 = r[0] * a0 + r[1] * a1 + r[2] * a2;
  int b1 = r[3] * a0 + r[4] * a1 + r[5] * a2;
  int b2 = r[6] * a0 + r[7] * a1 + r[8] * a2;
  const int* ml = C.lf_miller + 3 * g;
  const int* m0 = C.miller + 3 * iG0;
  b0 += ml[0] + m0[0];
  b1 += ml[1] + m0[1];
  b2 += ml[2] + m0[2];
  const int* ri = C.RIc + 9 * R2;
  int c0 = ri[0] * b0 + ri[1] * b1 + ri[2] * b2 - C.box_lo0;
  int c1 = ri[3] * b0 + ri[4] * b1 + ri[5] * b2 - C.box_lo1;
  int c2 = ri[6] * b0 + ri[7] * b1 + ri[8] * b2 - C.box_lo2;
  if ((unsigned)c0 >= (unsigned)C.box_d0 || (unsigned)c1 >= (unsigned)C.box_d1 ||
      (unsigned)c2 >= (unsigned)C.box_d2)
    return -1;
  int gg = C.box[((size_t)c0 * C.box_d1 + c1) * C.box_d2 + c2];
  if (gg < 0) return -1;
  if (C.legacy) return gg < C.npw[K2] ? gg : -1;
  return C.inv[(size_t)K2 * C.ng + gg];
}

// Current-vertex factors 0.5*j_mu (Optabs.f90:1410-1423): component ca into
// f.x and cb into f.y.
__device__ __forceinline__ double2 current_factor(const MapCtx& C, const int* km, const double* kv, int g, int i,
                                                  int ca, int cb) {
  int K1 = km[0], R1 = km[1];
  int gi = C.gidx[(size_t)K1 * C.npwx + i];
  const double* g1 = C.G + 3 * gi;
  const double* R = C.Rcart + 9 * R1;
  double k11 = R[0] * g1[0] + R[1] * g1[1] + R[2] * g1[2];
  double k22 = R[3] * g1[0] + R[4] * g1[1] + R[5] * g1[2];
  double k33 = R[6] * g1[0] + R[7] * g1[1] + R[8] * g1[2];
  const double* gl = C.Glf + 3 * g;
  double j[3];
  j[0] = (C.q0 + 2.0 * kv[0] + gl[0] + 2.0 * k11) * C.Gcar;
  j[1] = (C.q1 + 2.0 * kv[1] + gl[1] + 2.0 * k22) * C.Gcar;
  j[2] = (C.q2 + 2.0 * kv[2] + gl[2] + 2.0 * k33) * C.Gcar;
  return make_double2(0.5 * j[ca], 0.5 * j[cb]);
}

template <int IC, int MAXO, bool CURRENT, bool TWO>
__global__ void __launch_bounds__(256) k_vertex_fp64(MapCtx C, const double2* __restrict__ coeff,
                                                     const Trans* __restrict__ trans,
                                                     const long long* __restrict__ offsets, int k0, int GC,
                                                     int nbnd, int ca, int cb, double2* __restrict__ M,
                                                     double2* __restrict__ M2) {
  extern __shared__ double2 sm[];
  const int kl = blockIdx.x;
  const int ik = k0 + kl;
  const long long t0 = offsets[kl], t1 = offsets[kl + 1];
  const int P = (int)(t1 - t0);
  if (P == 0) return;
  const int g0 = blockIdx.y * GC;
  const int ng_here = min(GC, C.nlf - g0);
  if (ng_here <= 0) return;
  const int* km = C.kmap + 5 * ik;
  const int K1 = km[0], K2 = km[2];
  const int nsum = C.legacy ? C.nsum_legacy : C.npw[K1];
  const double* kv = C.ktot + 3 * ik;

  double2* C1s = sm;                               // [IC][nbnd]
  double2* C2s = C1s + IC * nbnd;                  // [GC][IC][nbnd]
  double2* C2b = C2s + (size_t)GC * IC * nbnd;     // second component (TWO)
  int* pos_s = reinterpret_cast<int*>(C2b + (TWO ? (size_t)GC * IC * nbnd : 0));  // [GC][IC]
  double2* fac_s = reinterpret_cast<double2*>(pos_s + ((GC * IC + 1) & ~1));       // [GC][IC]

  // outputs of this thread: o = tid + 256*u  ->  (transition o / ng_here, field o % ng_here)
  const int nout = P * ng_here;
  double2 acc[MAXO], acc2[MAXO];
  int on[MAXO], om[MAXO];
#pragma unroll
  for (int u = 0; u < MAXO; ++u) {
    acc[u] = make_double2(0.0, 0.0);
    acc2[u] = make_double2(0.0, 0.0);
    int o = threadIdx.x + 256 * u;
    if (o < nout) {
      int nm = trans[t0 + o / ng_here].nm;
      on[u] = nm & 0xffff;
      om[u] = ((o % ng_here) * IC) * nbnd + (nm >> 16);  // offset of (g, ii=0, m) in C2s
    } else {
      on[u] = 0;
      om[u] = -1;
    }
  }

  for (int i0 = 0; i0 < nsum; i0 += IC) {
    __syncthreads();
    for (int e = threadIdx.x; e < ng_here * IC; e += 256) {
      int g = e / IC, ii = e % IC, i = i0 + ii;
      int pos = -1;
      double2 f = make_double2(1.0, 1.0);
      if (i < nsum) {
        pos = gfast_pos(C, km, g0 + g, i);
        if (CURRENT) f = current_factor(C, km, kv, g0 + g, i, ca, cb);
      }
      pos_s[e] = pos;
      fac_s[e] = f;
    }
    for (int e = threadIdx.x; e < IC * nbnd; e += 256) {
      int ii = e / nbnd, b = e % nbnd, i = i0 + ii;
      C1s[e] = i < nsum ? coeff[((size_t)K1 * C.npwx + i) * nbnd + b] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < ng_here * IC * nbnd; e += 256) {
      int gi = e / nbnd, b = e % nbnd;
      int pos = pos_s[gi];
      double2 v = pos >= 0 ? coeff[((size_t)K2 * C.npwx + pos) * nbnd + b] : make_double2(0.0, 0.0);
      if (CURRENT) {
        double2 f = fac_s[gi];
        C2s[e] = make_double2(v.x * f.x, v.y * f.x);
        if (TWO) C2b[e] = make_double2(v.x * f.y, v.y * f.y);
      } else {
        C2s[e] = v;
      }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < MAXO; ++u) {
      if (om[u] < 0) continue;
      const double2* c1 = C1s + on[u];
      const double2* c2 = C2s + om[u];
      const double2* c2b = C2b + om[u];
      double ar = acc[u].x, ai = acc[u].y, br = acc2[u].x, bi = acc2[u].y;
#pragma unroll 4
      for (int ii = 0; ii < IC; ++ii) {
        double2 a = c1[ii * nbnd];
        double2 b = c2[ii * nbnd];
        // conj(a) * b
        ar = fma(a.x, b.x, ar);
        ar = fma(a.y, b.y, ar);
        ai = fma(a.x, b.y, ai);
        ai = fma(-a.y, b.x, ai);
        if (TWO) {
          double2 d = c2b[ii * nbnd];
          br = fma(a.x, d.x, br);
          br = fma(a.y, d.y, br);
          bi = fma(a.x, d.y, bi);
          bi = fma(-a.y, d.x, bi);
        }
      }
      acc[u] = make_double2(ar, ai);
      acc2[u] = make_double2(br, bi);
    }
  }
#pragma unroll
  for (int u = 0; u < MAXO; ++u) {
    int o = threadIdx.x + 256 * u;
    if (o >= nout) continue;
    long long t = t0 + o / ng_here;
    int g = g0 + o % ng_here;
    M[t * C.nlf + g] = acc[u];
    if (TWO) M2[t * C.nlf + g] = acc2[u];
  }
}

// ---------------------------------------------------------------------------
// Mixed path: FP32 complex coefficients, FP32 sums over slices of IC
// coefficients carried in double-float (hi + lo) across slices, result
// written as complex64 straight into the window-sorted row pos[t] that the
// tensor-core accumulation reads.  amax collects max |Re|, |Im| (float bits).
__device__ __forceinline__ void df_acc(float& hi, float& lo, float v) {
  float s = hi + v;
  float bb = s - hi;
  float e = (hi - (s - bb)) + (v - bb);
  lo += e;
  float h = s + lo;
  lo = lo - (h - s);
  hi = h;
}

template <int IC, int MAXO, bool CURRENT, bool TWO>
__global__ void __launch_bounds__(256) k_vertex_f32(MapCtx C, const float2* __restrict__ coeff,
                                                    const Trans* __restrict__ trans,
                                                    const long long* __restrict__ offsets,
                                                    const int* __restrict__ pos_of, int k0, int GC, int nbnd,
                                                    int ca, int cb, float2* __restrict__ M, float2* __restrict__ M2,
                                                    unsigned* __restrict__ amax) {
  extern __shared__ float2 smf[];
  const int kl = blockIdx.x;
  const int ik = k0 + kl;
  const long long t0 = offsets[kl], t1 = offsets[kl + 1];
  const int P = (int)(t1 - t0);
  if (P == 0) return;
  const int g0 = blockIdx.y * GC;
  const int ng_here = min(GC, C.nlf - g0);
  if (ng_here <= 0) return;
  const int* km = C.kmap + 5 * ik;
  const int K1 = km[0], K2 = km[2];
  const int nsum = C.legacy ? C.nsum_legacy : C.npw[K1];
  const double* kv = C.ktot + 3 * ik;

  float2* C1s = smf;                               // [IC][nbnd]
  float2* C2s = C1s + IC * nbnd;                   // [GC][IC][nbnd]
  float2* C2b = C2s + (size_t)GC * IC * nbnd;      // second component (TWO)
  int* pos_s = reinterpret_cast<int*>(C2b + (TWO ? (size_t)GC * IC * nbnd : 0));  // [GC][IC]
  float2* fac_s = reinterpret_cast<float2*>(pos_s + GC * IC);                     // [GC][IC]

  const int nout = P * ng_here;
  float ahr[MAXO], alr[MAXO], ahi[MAXO], ali[MAXO];
  float bhr[MAXO], blr[MAXO], bhi[MAXO], bli[MAXO];
  int on[MAXO], om[MAXO];
#pragma unroll
  for (int u = 0; u < MAXO; ++u) {
    ahr[u] = alr[u] = ahi[u] = ali[u] = bhr[u] = blr[u] = bhi[u] = bli[u] = 0.f;
    int o = threadIdx.x + 256 * u;
    if (o < nout) {
      int nm = trans[t0 + o / ng_here].nm;
      on[u] = nm & 0xffff;
      om[u] = ((o % ng_here) * IC) * nbnd + (nm >> 16);
    } else {
      on[u] = 0;
      om[u] = -1;
    }
  }

  for (int i0 = 0; i0 < nsum; i0 += IC) {
    __syncthreads();
    for (int e = threadIdx.x; e < ng_here * IC; e += 256) {
      int g = e / IC, ii = e % IC, i = i0 + ii;
      int pos = -1;
      float2 f = make_float2(1.f, 1.f);
      if (i < nsum) {
        pos = gfast_pos(C, km, g0 + g, i);
        if (CURRENT) {
          double2 fd = current_factor(C, km, kv, g0 + g, i, ca, cb);
          f = make_float2((float)fd.x, (float)fd.y);
        }
      }
      pos_s[e] = pos;
      fac_s[e] = f;
    }
    for (int e = threadIdx.x; e < IC * nbnd; e += 256) {
      int ii = e / nbnd, b = e % nbnd, i = i0 + ii;
      C1s[e] = i < nsum ? coeff[((size_t)K1 * C.npwx + i) * nbnd + b] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < ng_here * IC * nbnd; e += 256) {
      int gi = e / nbnd, b = e % nbnd;
      int pos = pos_s[gi];
      float2 v = pos >= 0 ? coeff[((size_t)K2 * C.npwx + pos) * nbnd + b] : make_float2(0.f, 0.f);
      if (CURRENT) {
        float2 f = fac_s[gi];
        C2s[e] = make_float2(v.x * f.x, v.y * f.x);
        if (TWO) C2b[e] = make_float2(v.x * f.y, v.y * f.y);
      } else {
        C2s[e] = v;
      }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < MAXO; ++u) {
      if (om[u] < 0) continue;
      const float2* c1 = C1s + on[u];
      const float2* c2 = C2s + om[u];
      const float2* c2b = C2b + om[u];
      float ar = 0.f, ai = 0.f, br = 0.f, bi = 0.f;
#pragma unroll 8
      for (int ii = 0; ii < IC; ++ii) {
        float2 a = c1[ii * nbnd];
        float2 b = c2[ii * nbnd];
        ar = fmaf(a.x, b.x, ar);
        ar = fmaf(a.y, b.y, ar);
        ai = fmaf(a.x, b.y, ai);
        ai = fmaf(-a.y, b.x, ai);
        if (TWO) {
          float2 d = c2b[ii * nbnd];
          br = fmaf(a.x, d.x, br);
          br = fmaf(a.y, d.y, br);
          bi = fmaf(a.x, d.y, bi);
          bi = fmaf(-a.y, d.x, bi);
        }
      }
      df_acc(ahr[u], alr[u], ar);
      df_acc(ahi[u], ali[u], ai);
      if (TWO) {
        df_acc(bhr[u], blr[u], br);
        df_acc(bhi[u], bli[u], bi);
      }
    }
  }
  float mx = 0.f, mx2 = 0.f;
#pragma unroll
  for (int u = 0; u < MAXO; ++u) {
    int o = threadIdx.x + 256 * u;
    if (o >= nout) continue;
    long long t = t0 + o / ng_here;
    int g = g0 + o % ng_here;
    size_t row = (size_t)pos_of[t];
    float2 v = make_float2(ahr[u] + alr[u], ahi[u] + ali[u]);
    M[row * C.nlf + g] = v;
    mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
    if (TWO) {
      float2 w = make_float2(bhr[u] + blr[u], bhi[u] + bli[u]);
      M2[row * C.nlf + g] = w;
      mx2 = fmaxf(mx2, fmaxf(fabsf(w.x), fabsf(w.y)));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    mx2 = fmaxf(mx2, __shfl_xor_sync(0xffffffffu, mx2, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(amax, __float_as_uint(mx));
    if (TWO) atomicMax(amax + 1, __float_as_uint(mx2));
  }
}

MapCtx make_map_ctx(rpa_ctx* c) {
  MapCtx C;
  C.kmap = c->d_kmap.as<int>();
  C.ktot = c->d_ktot.as<double>();
  C.miller = c->d_miller.as<int>();
  C.G = c->d_G.as<double>();
  C.box = c->d_box.as<int>();
  C.box_lo0 = c->box_lo[0];
  C.box_lo1 = c->box_lo[1];
  C.box_lo2 = c->box_lo[2];
  C.box_d0 = c->box_dim[0];
  C.box_d1 = c->box_dim[1];
  C.box_d2 = c->box_dim[2];
  C.Rc = c->d_Rc.as<int>();
  C.RIc = c->d_RIc.as<int>();
  C.Rcart = c->d_Rcart.as<double>();
  C.npw = c->d_npw.as<int>();
  C.gidx = c->d_gidx.as<int>();
  C.inv = c->legacy ? nullptr : c->d_inv.as<int>();
  C.npwx = c->npwx;
  C.ng = c->ng;
  C.legacy = c->legacy ? 1 : 0;
  C.nsum_legacy = 0;
  C.lf_miller = c->d_lf_miller.as<int>();
  C.Glf = c->d_Glf.as<double>();
  C.nlf = c->nlf;
  C.q0 = c->q[0];
  C.q1 = c->q[1];
  C.q2 = c->q[2];
  C.Gcar = 0.0;
  return C;
}

// Vertices of the n_trans transitions emitted for FBZ k-points [k0, k0+nk).
int vertices_fp64(rpa_ctx* c, const Chi0Plan& P, int k0, int nk, int maxpairs, long long n_trans) {
  const bool current = P.mode == RPA_MODE_CURRENT;
  const bool two = current && (P.pol == RPA_POL_YZ || P.pol == RPA_POL_ZY);
  RPA_TRY(ensure(c, c->d_M, sizeof(double2) * (size_t)(n_trans + 1) * c->nlf));
  if (two) RPA_TRY(ensure(c, c->d_M2, sizeof(double2) * (size_t)(n_trans + 1) * c->nlf));
  if (n_trans == 0) return RPA_OK;
  MapCtx C = make_map_ctx(c);
  C.nsum_legacy = P.nsum_legacy;
  C.Gcar = P.Gcar;
  constexpr int IC = 16, MAXO = 8;
  int GC = maxpairs > 0 ? (MAXO * 256) / maxpairs : 1;
  GC = GC < 1 ? 1 : (GC > 16 ? 16 : GC);
  if (GC > c->nlf) GC = c->nlf;
  if (maxpairs * GC > MAXO * 256) return fail(c, RPA_EINVAL, "too many band pairs per k-point (%d)", maxpairs);
  int ca = 0, cb = 0;
  switch (P.pol) {
    case RPA_POL_XX: ca = cb = 0; break;
    case RPA_POL_YY: ca = cb = 1; break;
    case RPA_POL_ZZ: ca = cb = 2; break;
    case RPA_POL_YZ: ca = 1; cb = 2; break;
    default: ca = 2; cb = 1; break;
  }
  size_t smem = sizeof(double2) * ((size_t)IC * c->nbnd + (size_t)GC * IC * c->nbnd * (two ? 2 : 1)) +
                sizeof(int) * (((size_t)GC * IC + 1) & ~(size_t)1) + sizeof(double2) * (size_t)GC * IC;
  dim3 grid(nk, (c->nlf + GC - 1) / GC);
  double2* M = c->d_M.as<double2>();
  double2* M2 = two ? c->d_M2.as<double2>() : M;
  const double2* coeff = c->d_coeff.as<double2>();
  const Trans* tr = c->d_trans.as<Trans>();
  const long long* off = c->d_offsets.as<long long>();
  if (!current) {
    auto kern = k_vertex_fp64<IC, MAXO, false, false>;
    RPA_CUDA(c, allow_dynamic_smem(kern, c->device));
    kern<<<grid, 256, smem, c->stream>>>(C, coeff, tr, off, k0, GC, c->nbnd, ca, cb, M, M2);
  } else if (!two) {
    auto kern = k_vertex_fp64<IC, MAXO, true, false>;
    RPA_CUDA(c, allow_dynamic_smem(kern, c->device));
    kern<<<grid, 256, smem, c->stream>>>(C, coeff, tr, off, k0, GC, c->nbnd, ca, cb, M, M2);
  } else {
    auto kern = k_vertex_fp64<IC, MAXO, true, true>;
    RPA_CUDA(c, allow_dynamic_smem(kern, c->device));
    kern<<<grid, 256, smem, c->stream>>>(C, coeff, tr, off, k0, GC, c->nbnd, ca, cb, M, M2);
  }
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

// Mixed-path vertices of the n_trans transitions of FBZ k-points [k0, k0+nk),
// written to rows pos_of[t] of Mf (and Mf2).
int vertices_f32(rpa_ctx* c, const Chi0Plan& P, int k0, int nk, int maxpairs, long long n_trans, const int* pos_of,
                 float2* Mf, float2* Mf2, unsigned* amax) {
  if (n_trans == 0) return RPA_OK;
  const bool current = P.mode == RPA_MODE_CURRENT;
  const bool two = current && (P.pol == RPA_POL_YZ || P.pol == RPA_POL_ZY);
  MapCtx C = make_map_ctx(c);
  C.nsum_legacy = P.nsum_legacy;
  C.Gcar = P.Gcar;
  constexpr int IC = 32, MAXO = 8;
  int GC = maxpairs > 0 ? (MAXO * 256) / maxpairs : 1;
  GC = GC < 1 ? 1 : (GC > 16 ? 16 : GC);
  if (GC > c->nlf) GC = c->nlf;
  if (maxpairs * GC > MAXO * 256) return fail(c, RPA_EINVAL, "too many band pairs per k-point (%d)", maxpairs);
  int ca = 0, cb = 0;
  switch (P.pol) {
    case RPA_POL_XX: ca = cb = 0; break;
    case RPA_POL_YY: ca = cb = 1; break;
    case RPA_POL_ZZ: ca = cb = 2; break;
    case RPA_POL_YZ: ca = 1; cb = 2; break;
    default: ca = 2; cb = 1; break;
  }
  size_t smem = sizeof(float2) * ((size_t)IC * c->nbnd + (size_t)GC * IC * c->nbnd * (two ? 2 : 1)) +
                sizeof(int) * (size_t)GC * IC + sizeof(float2) * (size_t)GC * IC;
  dim3 grid(nk, (c->nlf + GC - 1) / GC);
  if (!c->d_coeff32.p) return fail(c, RPA_ESTATE, "FP32 vertices: no FP32 copy of the basis on the device");
  const float2* coeff = c->d_coeff32.as<float2>();
  const Trans* tr = c->d_trans.as<Trans>();
  const long long* off = c->d_offsets.as<long long>();
  if (!current) {
    auto kern = k_vertex_f32<IC, MAXO, false, false>;
    RPA_CUDA(c, allow_dynamic_smem(kern, c->device));
    kern<<<grid, 256, smem, c->stream>>>(C, coeff, tr, off, pos_of, k0, GC, c->nbnd, ca, cb, Mf, Mf, amax);
  } else if (!two) {
    auto kern = k_vertex_f32<IC, MAXO, true, false>;
    RPA_CUDA(c, allow_dynamic_smem(kern, c->device));
    kern<<<grid, 256, smem, c->stream>>>(C, coeff, tr, off, pos_of, k0, GC, c->nbnd, ca, cb, Mf, Mf, amax);
  } else {
    auto kern = k_vertex_f32<IC, MAXO, true, true>;
    RPA_CUDA(c, allow_dynamic_smem(kern, c->device));
    kern<<<grid, 256, smem, c->stream>>>(C, coeff, tr, off, pos_of, k0, GC, c->nbnd, ca, cb, Mf, Mf2, amax);
  }
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

// Gfast maps, one block per FBZ k-point.  The box coordinate of a pair
// separates, c(G, i) = base(i) + shift(G):
//   forward  base(i) = RI2 (R1 G_i + G_iG0) - lo,    shift(G) = RI2 Glf_G
//   inverse  base(p) = RI1 (R2 G_p - G_iG0) - lo,    shift(G) = -RI1 Glf_G
// (i a plane wave of K1, p one of K2; gfast_pos / gfast_inv_pos give the same
// positions element by element), so both tables go to shared memory and every
// (G, i) is one add, a bounds test, the box lookup and the basis lookup.
// out[k_local][G][i] for i < nsum_max, -1 where absent or beyond the basis.
template <bool INV>
__global__ void __launch_bounds__(512) k_map_k(MapCtx C, int k0, int nsum_max, int16_t* __restrict__ out) {
  extern __shared__ int msm[];
  int* base = msm;                   // [3][nsum_max]
  int* shift = msm + 3 * nsum_max;   // [3][nlf]
  const int kl = blockIdx.x;
  const int* km = C.kmap + 5 * (k0 + kl);
  const int K1 = km[0], R1 = km[1], K2 = km[2], R2 = km[3], iG0 = km[4];
  const int kS = INV ? K2 : K1;  // basis of the summed index
  const int kL = INV ? K1 : K2;  // basis the positions refer to
  const int ns = INV ? C.npw[K2] : (C.legacy ? C.nsum_legacy : C.npw[K1]);
  const int* r = C.Rc + 9 * (INV ? R2 : R1);
  const int* ri = C.RIc + 9 * (INV ? R1 : R2);
  const int* m0 = C.miller + 3 * iG0;
  const int sg = INV ? -1 : 1;
  for (int i = threadIdx.x; i < nsum_max; i += blockDim.x) {
    int c0 = 0, c1 = 0, c2 = 0;
    if (i < ns) {
      const int* m = C.miller + 3 * C.gidx[(size_t)kS * C.npwx + i];
      const int b0 = r[0] * m[0] + r[1] * m[1] + r[2] * m[2] + sg * m0[0];
      const int b1 = r[3] * m[0] + r[4] * m[1] + r[5] * m[2] + sg * m0[1];
      const int b2 = r[6] * m[0] + r[7] * m[1] + r[8] * m[2] + sg * m0[2];
      c0 = ri[0] * b0 + ri[1] * b1 + ri[2] * b2 - C.box_lo0;
      c1 = ri[3] * b0 + ri[4] * b1 + ri[5] * b2 - C.box_lo1;
      c2 = ri[6] * b0 + ri[7] * b1 + ri[8] * b2 - C.box_lo2;
    } else {
      c0 = INT_MIN / 2;  // outside the box for every shift
    }
    base[i] = c0;
    base[nsum_max + i] = c1;
    base[2 * nsum_max + i] = c2;
  }
  for (int g = threadIdx.x; g < C.nlf; g += blockDim.x) {
    const int* ml = C.lf_miller + 3 * g;
    shift[g] = sg * (ri[0] * ml[0] + ri[1] * ml[1] + ri[2] * ml[2]);
    shift[C.nlf + g] = sg * (ri[3] * ml[0] + ri[4] * ml[1] + ri[5] * ml[2]);
    shift[2 * C.nlf + g] = sg * (ri[6] * ml[0] + ri[7] * ml[1] + ri[8] * ml[2]);
  }
  __syncthreads();
  const int* inv = C.inv + (size_t)kL * C.ng;
  const int nposL = C.npw[kL];
  int16_t* o = out + (size_t)kl * C.nlf * nsum_max;
  for (int g = 0; g < C.nlf; ++g) {
    const int s0 = shift[g], s1 = shift[C.nlf + g], s2 = shift[2 * C.nlf + g];
    for (int i = threadIdx.x; i < nsum_max; i += blockDim.x) {
      const int c0 = base[i] + s0, c1 = base[nsum_max + i] + s1, c2 = base[2 * nsum_max + i] + s2;
      int pos = -1;
      if ((unsigned)c0 < (unsigned)C.box_d0 && (unsigned)c1 < (unsigned)C.box_d1 && (unsigned)c2 < (unsigned)C.box_d2) {
        const int gg = C.box[((size_t)c0 * C.box_d1 + c1) * C.box_d2 + c2];
        if (gg >= 0) pos = (C.legacy && !INV) ? (gg < nposL ? gg : -1) : inv[gg];
      }
      o[(size_t)g * nsum_max + i] = (int16_t)pos;
    }
  }
}

static bool map_k_fits(const rpa_ctx* c, int nsum_max) {
  return (size_t)(3 * nsum_max + 3 * c->nlf) * sizeof(int) <= (size_t)160 << 10;
}

template <bool INV>
static int launch_map_k(rpa_ctx* c, const MapCtx& C, int k0, int nk, int nsum_max, int16_t* out) {
  const size_t smem = (size_t)(3 * nsum_max + 3 * c->nlf) * sizeof(int);
  RPA_CUDA(c, allow_dynamic_smem(k_map_k<INV>, c->device));
  k_map_k<INV><<<nk, 512, smem, c->stream>>>(C, k0, nsum_max, out);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

// Gfast maps of the FBZ k-points [k0, k0+nk) as int16 basis positions
// (-1 absent), gmap[k_local][G][i] for i < nsum_max (-1 beyond nsum).
__global__ void k_gmap(MapCtx C, int k0, int nk, int nsum_max, int16_t* __restrict__ gmap) {
  const size_t per_k = (size_t)C.nlf * nsum_max;
  const size_t n = (size_t)nk * per_k;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    int kl = (int)(e / per_k);
    size_t r = e % per_k;
    int g = (int)(r / nsum_max), i = (int)(r % nsum_max);
    const int* km = C.kmap + 5 * (k0 + kl);
    int nsum = C.legacy ? C.nsum_legacy : C.npw[km[0]];
    gmap[e] = (int16_t)(i < nsum ? gfast_pos(C, km, g, i) : -1);
  }
}

int build_gmap(rpa_ctx* c, int k0, int nk, int nsum_max, int16_t* gmap, int nsum_legacy) {
  MapCtx C = make_map_ctx(c);
  C.nsum_legacy = nsum_legacy;
  if (map_k_fits(c, nsum_max)) return launch_map_k<false>(c, C, k0, nk, nsum_max, gmap);
  k_gmap<<<4096, 256, 0, c->stream>>>(C, k0, nk, nsum_max, gmap);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

// Basis position in K1 of the plane wave that Gfast sends to basis position p
// of K2 for local field g, or -1: Gfast inverted in integer crystal
// coordinates, G_i = R1^-1 (R2 G_p - Glf_g - G_iG0), then looked up in K1's basis.
__device__ __forceinline__ int gfast_inv_pos(const MapCtx& C, const int* km, int g, int p) {
  int K1 = km[0], R1 = km[1], K2 = km[2], R2 = km[3], iG0 = km[4];
  int gp = C.gidx[(size_t)K2 * C.npwx + p];
  const int* mp = C.miller + 3 * gp;
  const int* r = C.Rc + 9 * R2;
  int b0 = r[0] * mp[0] + r[1] * mp[1] + r[2] * mp[2];
  int b1 = r[3] * mp[0] + r[4] * mp[1] + r[5] * mp[2];
  int b2 = r[6] * mp[0] + r[7] * mp[1] + r[8] * mp[2];
  const int* ml = C.lf_miller + 3 * g;
  const int* m0 = C.miller + 3 * iG0;
  b0 -= ml[0] + m0[0];
  b1 -= ml[1] + m0[1];
  b2 -= ml[2] + m0[2];
  const int* ri = C.RIc + 9 * R1;
  int c0 = ri[0] * b0 + ri[1] * b1 + ri[2] * b2 - C.box_lo0;
  int c1 = ri[3] * b0 + ri[4] * b1 + ri[5] * b2 - C.box_lo1;
  int c2 = ri[6] * b0 + ri[7] * b1 + ri[8] * b2 - C.box_lo2;
  if ((unsigned)c0 >= (unsigned)C.box_d0 || (unsigned)c1 >= (unsigned)C.box_d1 ||
      (unsigned)c2 >= (unsigned)C.box_d2)
    return -1;
  int gg = C.box[((size_t)c0 * C.box_d1 + c1) * C.box_d2 + c2];
  if (gg < 0) return -1;
  return C.inv[(size_t)K1 * C.ng + gg];
}

// Inverse maps of the FBZ k-points [k0, k0+nk): ginv[k_local][G][p] = the K1
// plane wave i with Gfast(G, i) = p (a basis position of K2), -1 where none or
// p >= npw(K2).  Gfast(G, .) is injective (distinct G_i give distinct G''), and
// R1, R2 are unimodular integer matrices in crystal coordinates, so the inverse
// is computed directly for every p (one coalesced write each) and agrees with
// inverting the forward map.
__global__ void k_ginv(MapCtx C, int k0, int nk, int nsum_max, int16_t* __restrict__ ginv) {
  const size_t per_k = (size_t)C.nlf * nsum_max;
  const size_t n = (size_t)nk * per_k;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int kl = (int)(e / per_k);
    const size_t r = e % per_k;
    const int g = (int)(r / nsum_max), p = (int)(r % nsum_max);
    const int* km = C.kmap + 5 * (k0 + kl);
    ginv[e] = (int16_t)(p < C.npw[km[2]] ? gfast_inv_pos(C, km, g, p) : -1);
  }
}

int build_ginv(rpa_ctx* c, int k0, int nk, int nsum_max, int16_t* ginv) {
  if (c->legacy) return fail(c, RPA_EINVAL, "inverse Gfast map: needs the igk map of the basis");
  MapCtx C = make_map_ctx(c);
  if (map_k_fits(c, nsum_max)) return launch_map_k<true>(c, C, k0, nk, nsum_max, ginv);
  k_ginv<<<4096, 256, 0, c->stream>>>(C, k0, nk, nsum_max, ginv);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

// Gfast map of one FBZ k-point in the reference's convention (1-based basis
// positions, NG2+1 when absent), for the index-map parity checks.
__global__ void k_gfast(MapCtx C, int ik, int nsum, int* out) {
  const int* km = C.kmap + 5 * ik;
  int NG2 = C.npw[km[2]];
  int n = C.nlf * nsum;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    int g = e / nsum, i = e % nsum;
    int pos = gfast_pos(C, km, g, i);
    out[e] = pos >= 0 ? pos + 1 : NG2 + 1;
  }
}

int build_gfast(rpa_ctx* c, int ik, int nsum_legacy, int* host_out) {
  MapCtx C = make_map_ctx(c);
  int K1 = c->h_kmap[5 * ik];
  int nsum = c->legacy ? nsum_legacy : c->h_npw[K1];
  size_t n = (size_t)c->nlf * nsum;
  RPA_TRY(ensure(c, c->d_tmp, sizeof(int) * (n + 1)));
  k_gfast<<<(int)((n + 255) / 256), 256, 0, c->stream>>>(C, ik, nsum, c->d_tmp.as<int>());
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  RPA_CUDA(c, cudaMemcpyAsync(host_out, c->d_tmp.p, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  return RPA_OK;
}

}  // namespace rpa
