// k_kmap.cu -- the k-point bookkeeping of the drivers on the device: the full
// Brillouin zone from the IBZ and the point group (genFBZ,
// Chi_RPA/Optabs.f90:886-933), the IBZ point and symmetry of every FBZ point
// (findKinIBZ, Optabs.f90:776-818) and of every K+Q (findKQinBZ,
// Optabs.f90:820-884).  Results are identical to the reference's loops:
//  - genFBZ: candidate c = (symmetry i, IBZ point j), i outer, is kept unless an
//    earlier candidate lies within eps in every component;
//  - findKinIBZ: FBZ points 1..NkI are their own IBZ points (R1 = 1); later
//    ones take the first symmetry i >= 2, then the first IBZ point j, with
//    |RI_i k - kI_j| <= eps;
//  - findKQinBZ: the first G (list order), then the first FBZ point jk, with
//    |K+Q - G - ktot_jk| <= eps and an IBZ match for ktot_jk (first symmetry
//    from 1, first IBZ point).  At most one G can match a given (K+Q, jk) (G
//    vectors are a lattice spacing apart, eps is far below it), so the G of
//    each jk is found by rounding the crystal coordinates of K+Q - ktot_jk and
//    looking them up in the Miller box table, then confirmed with the
//    reference's own test; the answer is the smallest (G index, jk) pair that
//    passes.
// Products and sums are rounded one by one (no contraction), in the order of
// the Fortran expressions, so the eps comparisons see the reference's values.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "rpa_internal.cuh"

namespace rpa {

namespace {

struct Sym {
  double R[48][9];   // R(i, n, m) as [i][3 n + m]
  double RI[48][9];
};

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// k(n) = 0; do m: k(n) = k(n) + R(i,n,m) kI(m)   (genFBZ)
__global__ void k_fbz_candidates(Sym S, const double* __restrict__ kI, int nsym, int nki, double* __restrict__ kc) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nsym * nki) return;
  const int i = c / nki, j = c % nki;
  for (int n = 0; n < 3; ++n) {
    double s = 0.0;
    for (int m = 0; m < 3; ++m) s = add(s, mul(S.R[i][3 * n + m], kI[3 * j + m]));
    kc[3 * c + n] = s;
  }
}

// keep[c] = no earlier candidate within eps in all three components; one warp per c
__global__ void k_fbz_dedup(const double* __restrict__ kc, int C, double eps, int* __restrict__ keep) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= C) return;
  const double x = kc[3 * warp], y = kc[3 * warp + 1], z = kc[3 * warp + 2];
  bool dup = false;
  for (int base = 0; base < warp && !dup; base += 32) {
    const int l = base + lane;
    bool d = false;
    if (l < warp)
      d = fabs(sub(x, kc[3 * l])) <= eps && fabs(sub(y, kc[3 * l + 1])) <= eps && fabs(sub(z, kc[3 * l + 2])) <= eps;
    dup = __any_sync(0xffffffffu, d);
  }
  if (lane == 0) keep[warp] = dup ? 0 : 1;
}

// first IBZ point j (0-based) with |K - kI_j| <= eps, -1 if none; lanes scan j in order
__device__ int first_ibz(const double* __restrict__ kI, int nki, double K1, double K2, double K3, double eps,
                         int lane) {
  for (int base = 0; base < nki; base += 32) {
    const int j = base + lane;
    const bool m = j < nki && fabs(sub(K1, kI[3 * j])) <= eps && fabs(sub(K2, kI[3 * j + 1])) <= eps &&
                   fabs(sub(K3, kI[3 * j + 2])) <= eps;
    const unsigned b = __ballot_sync(0xffffffffu, m);
    if (b) return base + __ffs(b) - 1;
  }
  return -1;
}

// K = RI_i k as RI(i,n,1) kx + RI(i,n,2) ky + RI(i,n,3) kz (left to right)
__device__ __forceinline__ void rot(const double* r, double kx, double ky, double kz, double& a, double& b,
                                    double& c) {
  a = add(add(mul(r[0], kx), mul(r[1], ky)), mul(r[2], kz));
  b = add(add(mul(r[3], kx), mul(r[4], ky)), mul(r[5], kz));
  c = add(add(mul(r[6], kx), mul(r[7], ky)), mul(r[8], kz));
}

// findKinIBZ for FBZ points nki..ntot-1 (0-based); one warp per point
__global__ void k_find_k_ibz(Sym S, const double* __restrict__ ktot, const double* __restrict__ kI, int ntot, int nki,
                             int nsym, double eps, int* __restrict__ R1, int* __restrict__ K1) {
  const int ik = nki + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (ik >= ntot) return;
  const double kx = ktot[3 * ik], ky = ktot[3 * ik + 1], kz = ktot[3 * ik + 2];
  for (int i = 1; i < nsym; ++i) {
    double a, b, c;
    rot(S.RI[i], kx, ky, kz, a, b, c);
    const int j = first_ibz(kI, nki, a, b, c, eps, lane);
    if (j >= 0) {
      if (lane == 0) R1[ik] = i + 1, K1[ik] = j + 1;
      return;
    }
  }
  if (lane == 0) R1[ik] = 0, K1[ik] = 0;
}

struct KqCtx {
  const double* ktot;
  const double* kI;
  const double* G;     // [ng][3]
  const int* box;
  int box_lo0, box_lo1, box_lo2, box_d0, box_d1, box_d2;
  double KCi[9];       // Cartesian -> crystal (row-major)
  double q0, q1, q2, eps;
  int ntot, nki, nsym;
};

// findKQinBZ for every FBZ point; one warp per point
__global__ void k_find_kq(Sym S, KqCtx Q, int* __restrict__ iG0, int* __restrict__ R2, int* __restrict__ K2) {
  const int ik = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (ik >= Q.ntot) return;
  const double KQx = add(Q.ktot[3 * ik], Q.q0), KQy = add(Q.ktot[3 * ik + 1], Q.q1),
               KQz = add(Q.ktot[3 * ik + 2], Q.q2);
  long long best = -1;  // smallest passing key iG * ntot + jk
  for (int base = 0; base < Q.ntot; base += 32) {
    const int jk = base + lane;
    long long key = -1;
    if (jk < Q.ntot) {
      const double* kt = Q.ktot + 3 * jk;
      const double dx = KQx - kt[0], dy = KQy - kt[1], dz = KQz - kt[2];
      const double* M = Q.KCi;
      const long long m0 = llrint(M[0] * dx + M[1] * dy + M[2] * dz);
      const long long m1 = llrint(M[3] * dx + M[4] * dy + M[5] * dz);
      const long long m2 = llrint(M[6] * dx + M[7] * dy + M[8] * dz);
      const long long c0 = m0 - Q.box_lo0, c1 = m1 - Q.box_lo1, c2 = m2 - Q.box_lo2;
      if (c0 >= 0 && c0 < Q.box_d0 && c1 >= 0 && c1 < Q.box_d1 && c2 >= 0 && c2 < Q.box_d2) {
        const int g = Q.box[(c0 * Q.box_d1 + c1) * Q.box_d2 + c2];
        if (g >= 0) {
          const double* Gv = Q.G + 3 * g;
          if (fabs(sub(sub(KQx, Gv[0]), kt[0])) <= Q.eps && fabs(sub(sub(KQy, Gv[1]), kt[1])) <= Q.eps &&
              fabs(sub(sub(KQz, Gv[2]), kt[2])) <= Q.eps)
            key = (long long)g * Q.ntot + jk;
        }
      }
    }
    // this round's candidates one at a time (all lanes together); a candidate
    // counts when its FBZ point has an IBZ image and its key is the smallest so far
    unsigned cm = __ballot_sync(0xffffffffu, key >= 0);
    while (cm) {
      const int src = __ffs(cm) - 1;
      cm &= cm - 1;
      const long long k = __shfl_sync(0xffffffffu, key, src);
      if (best >= 0 && k >= best) continue;
      const double* kt = Q.ktot + 3 * (k % Q.ntot);
      bool ok = false;
      for (int i = 0; i < Q.nsym && !ok; ++i) {
        double a, b, c;
        rot(S.RI[i], kt[0], kt[1], kt[2], a, b, c);
        ok = first_ibz(Q.kI, Q.nki, a, b, c, Q.eps, lane) >= 0;
      }
      if (ok) best = k;
    }
  }
  if (best < 0) {
    if (lane == 0) iG0[ik] = R2[ik] = K2[ik] = 0;
    return;
  }
  const int g = (int)(best / Q.ntot), jk = (int)(best % Q.ntot);
  const double* kt = Q.ktot + 3 * jk;
  for (int i = 0; i < Q.nsym; ++i) {
    double a, b, c;
    rot(S.RI[i], kt[0], kt[1], kt[2], a, b, c);
    const int j = first_ibz(Q.kI, Q.nki, a, b, c, Q.eps, lane);
    if (j >= 0) {
      if (lane == 0) iG0[ik] = g + 1, R2[ik] = i + 1, K2[ik] = j + 1;
      return;
    }
  }
}

Sym make_sym(const rpa_ctx* c) {
  Sym S;
  for (int i = 0; i < 48; ++i)
    for (int n = 0; n < 3; ++n)
      for (int m = 0; m < 3; ++m) {
        S.R[i][3 * n + m] = c->h_R[i + 48 * (n + 3 * m)];
        S.RI[i][3 * n + m] = c->h_RI[i + 48 * (n + 3 * m)];
      }
  return S;
}

}  // namespace
}  // namespace rpa

using namespace rpa;

extern "C" {

int rpa_gen_fbz(rpa_ctx* c, int nki, const double* kI, double eps, int max_ntot, int* ntot, double* ktot) {
  if (!c || nki < 1 || !kI || !ntot || !ktot || max_ntot < 1 || !(eps >= 0))
    return fail(c, RPA_EINVAL, "rpa_gen_fbz: bad arguments");
  cudaSetDevice(c->device);
  const int C = c->nsym * nki;
  const Sym S = make_sym(c);
  DevBuf dk, dc, dkeep;
  RPA_TRY(ensure(c, dk, sizeof(double) * 3 * nki));
  RPA_TRY(ensure(c, dc, sizeof(double) * 3 * C));
  RPA_TRY(ensure(c, dkeep, sizeof(int) * C));
  int rc = RPA_OK;
  std::vector<double> kc(3 * (size_t)C);
  std::vector<int> keep(C);
  if (cudaMemcpyAsync(dk.p, kI, sizeof(double) * 3 * nki, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
    rc = fail(c, RPA_ECUDA, "rpa_gen_fbz: copy");
  if (rc == RPA_OK) {
    k_fbz_candidates<<<(C + 127) / 128, 128, 0, c->stream>>>(S, dk.as<double>(), c->nsym, nki, dc.as<double>());
    k_fbz_dedup<<<(C + 7) / 8, 256, 0, c->stream>>>(dc.as<double>(), C, eps, dkeep.as<int>());
    c->launches += 2;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(kc.data(), dc.p, sizeof(double) * 3 * C, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaMemcpyAsync(keep.data(), dkeep.p, sizeof(int) * C, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
      rc = fail(c, RPA_ECUDA, "rpa_gen_fbz: kernel");
  }
  release(dk);
  release(dc);
  release(dkeep);
  if (rc != RPA_OK) return rc;
  int n = 0;
  for (int e = 0; e < C; ++e) {
    if (!keep[e]) continue;
    if (n == max_ntot) return fail(c, RPA_EINVAL, "rpa_gen_fbz: more than max_ntot = %d FBZ points", max_ntot);
    std::copy(&kc[3 * (size_t)e], &kc[3 * (size_t)e] + 3, ktot + 3 * (size_t)n);
    ++n;
  }
  *ntot = n;
  return RPA_OK;
}

int rpa_find_k_ibz(rpa_ctx* c, int ntot, const double* ktot, int nki, const double* kI, double eps, int* R1,
                   int* K1) {
  if (!c || ntot < 1 || nki < 1 || nki > ntot || !ktot || !kI || !R1 || !K1 || !(eps >= 0))
    return fail(c, RPA_EINVAL, "rpa_find_k_ibz: bad arguments");
  cudaSetDevice(c->device);
  for (int ik = 0; ik < nki; ++ik) R1[ik] = 1, K1[ik] = ik + 1;
  if (ntot == nki) return RPA_OK;
  const Sym S = make_sym(c);
  DevBuf dt, dk, dr;
  int rc = RPA_OK;
  if ((rc = ensure(c, dt, sizeof(double) * 3 * ntot)) == RPA_OK && (rc = ensure(c, dk, sizeof(double) * 3 * nki)) == RPA_OK &&
      (rc = ensure(c, dr, sizeof(int) * 2 * ntot)) == RPA_OK) {
    int* dR = dr.as<int>();
    if (cudaMemcpyAsync(dt.p, ktot, sizeof(double) * 3 * ntot, cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
        cudaMemcpyAsync(dk.p, kI, sizeof(double) * 3 * nki, cudaMemcpyHostToDevice, c->stream) != cudaSuccess) {
      rc = fail(c, RPA_ECUDA, "rpa_find_k_ibz: copy");
    } else {
      const int nw = ntot - nki;
      k_find_k_ibz<<<(nw + 7) / 8, 256, 0, c->stream>>>(S, dt.as<double>(), dk.as<double>(), ntot, nki, c->nsym, eps,
                                                        dR, dR + ntot);
      ++c->launches;
      if (cudaGetLastError() != cudaSuccess ||
          cudaMemcpyAsync(R1 + nki, dR + nki, sizeof(int) * nw, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
          cudaMemcpyAsync(K1 + nki, dR + ntot + nki, sizeof(int) * nw, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
          cudaStreamSynchronize(c->stream) != cudaSuccess)
        rc = fail(c, RPA_ECUDA, "rpa_find_k_ibz: kernel");
    }
  }
  release(dt);
  release(dk);
  release(dr);
  if (rc != RPA_OK) return rc;
  for (int ik = nki; ik < ntot; ++ik)
    if (R1[ik] == 0) return fail(c, RPA_ENOTFOUND, "Can not find wave vector K=%d in I.B.Z.", ik + 1);
  return RPA_OK;
}

int rpa_find_kq(rpa_ctx* c, int ntot, const double* ktot, int nki, const double* kI, const double* q, double eps,
                int* iG0, int* R2, int* K2) {
  if (!c || ntot < 1 || nki < 1 || !ktot || !kI || !q || !iG0 || !R2 || !K2 || !(eps >= 0))
    return fail(c, RPA_EINVAL, "rpa_find_kq: bad arguments");
  if (c->ng == 0) return fail(c, RPA_ESTATE, "rpa_find_kq: no G vectors (call rpa_set_gvectors)");
  cudaSetDevice(c->device);
  const Sym S = make_sym(c);
  KqCtx Q;
  {
    double K[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) K[3 * i + j] = c->KC[i + 3 * j];
    const double det = K[0] * (K[4] * K[8] - K[5] * K[7]) - K[1] * (K[3] * K[8] - K[5] * K[6]) +
                       K[2] * (K[3] * K[7] - K[4] * K[6]);
    if (std::fabs(det) < 1e-14) return fail(c, RPA_EINVAL, "reciprocal axes KC are singular");
    double* Ki = Q.KCi;
    Ki[0] = (K[4] * K[8] - K[5] * K[7]) / det;
    Ki[1] = (K[2] * K[7] - K[1] * K[8]) / det;
    Ki[2] = (K[1] * K[5] - K[2] * K[4]) / det;
    Ki[3] = (K[5] * K[6] - K[3] * K[8]) / det;
    Ki[4] = (K[0] * K[8] - K[2] * K[6]) / det;
    Ki[5] = (K[2] * K[3] - K[0] * K[5]) / det;
    Ki[6] = (K[3] * K[7] - K[4] * K[6]) / det;
    Ki[7] = (K[1] * K[6] - K[0] * K[7]) / det;
    Ki[8] = (K[0] * K[4] - K[1] * K[3]) / det;
  }
  Q.G = c->d_G.as<double>();
  Q.box = c->d_box.as<int>();
  Q.box_lo0 = c->box_lo[0];
  Q.box_lo1 = c->box_lo[1];
  Q.box_lo2 = c->box_lo[2];
  Q.box_d0 = c->box_dim[0];
  Q.box_d1 = c->box_dim[1];
  Q.box_d2 = c->box_dim[2];
  Q.q0 = q[0];
  Q.q1 = q[1];
  Q.q2 = q[2];
  Q.eps = eps;
  Q.ntot = ntot;
  Q.nki = nki;
  Q.nsym = c->nsym;
  DevBuf dt, dk, dr;
  int rc = RPA_OK;
  if ((rc = ensure(c, dt, sizeof(double) * 3 * ntot)) == RPA_OK && (rc = ensure(c, dk, sizeof(double) * 3 * nki)) == RPA_OK &&
      (rc = ensure(c, dr, sizeof(int) * 3 * ntot)) == RPA_OK) {
    int* dR = dr.as<int>();
    Q.ktot = dt.as<double>();
    Q.kI = dk.as<double>();
    if (cudaMemcpyAsync(dt.p, ktot, sizeof(double) * 3 * ntot, cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
        cudaMemcpyAsync(dk.p, kI, sizeof(double) * 3 * nki, cudaMemcpyHostToDevice, c->stream) != cudaSuccess) {
      rc = fail(c, RPA_ECUDA, "rpa_find_kq: copy");
    } else {
      k_find_kq<<<(ntot + 7) / 8, 256, 0, c->stream>>>(S, Q, dR, dR + ntot, dR + 2 * ntot);
      ++c->launches;
      if (cudaGetLastError() != cudaSuccess ||
          cudaMemcpyAsync(iG0, dR, sizeof(int) * ntot, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
          cudaMemcpyAsync(R2, dR + ntot, sizeof(int) * ntot, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
          cudaMemcpyAsync(K2, dR + 2 * ntot, sizeof(int) * ntot, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
          cudaStreamSynchronize(c->stream) != cudaSuccess)
        rc = fail(c, RPA_ECUDA, "rpa_find_kq: kernel");
    }
  }
  release(dt);
  release(dk);
  release(dr);
  if (rc != RPA_OK) return rc;
  for (int ik = 0; ik < ntot; ++ik)
    if (iG0[ik] == 0) return fail(c, RPA_ENOTFOUND, "Can not find wave vector K+Q=%d+q in FBZ or IBZ.", ik + 1);
  return RPA_OK;
}

}  // extern "C"
