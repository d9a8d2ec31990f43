// k_accum.cu -- Lorentzian-weighted spectral accumulation, FP64 path.
//
// Reference: the S0 rank-1 updates of Sloss.f90:407-418 (real S0, io = 1..no)
// and Optabs.f90:387-421 (complex S0, io = -no..no), plus the intraband Qeff
// update Optabs.f90:430-443.  The reference applies, per transition t and per
// frequency io inside the Lorentzian window, S(io,G,G') += w(t,io) M(G) M2*(G').
//
// Here the transitions are sorted by window start, so the transitions that
// touch a block of BO frequency rows form one contiguous range.  A block owns
// a BO x (16 G x 8 G') tile of S in registers (one (G,G') pair per thread,
// BO complex accumulators), walks that range in slices of TT transitions,
// forms X = M(G) conj(M2(G')) once per transition and adds w X to every row
// of the tile inside the transition's window.  The window test is the exact
// predicate of k_setup.cu, so the set of (t, io) terms equals the reference's.

#include "rpa_internal.cuh"

namespace rpa {

struct AccCtx {
  const Trans* rec;   // sorted interband records (k := vertex row)
  const double2* M;
  const double2* M2;
  int nlf, nw, obase, wmax, n_inter;
  double domega, eta, cut_over_eta;
};

__device__ __forceinline__ double lorentz(const AccCtx& A, int r, double e1, double e2, bool* in) {
  double o = __dmul_rn((double)(r + A.obase), A.domega);
  double dE = __dadd_rn(__dadd_rn(o, e1), -e2);
  double den = __dadd_rn(__dmul_rn(dE, dE), __dmul_rn(A.eta, A.eta));
  double L = __ddiv_rn(A.eta, den);
  *in = L >= A.cut_over_eta;
  return L;
}

// First record whose window start is >= key (records sorted by lo).
__device__ int lower_bound_lo(const Trans* rec, int n, int key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (rec[mid].lo < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

template <int BO, int TT, bool CPLX>
__global__ void __launch_bounds__(128) k_accum_fp64(AccCtx A, double* __restrict__ S) {
  __shared__ double2 Ms[TT][16];
  __shared__ double2 M2s[TT][8];
  __shared__ double Ws[TT][BO];
  __shared__ int range[2];

  const int r0 = blockIdx.x * BO;
  const int gi0 = blockIdx.y * 16, gj0 = blockIdx.z * 8;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int gi = gi0 + tx, gj = gj0 + ty;

  if (threadIdx.x == 0) {
    range[0] = lower_bound_lo(A.rec, A.n_inter, r0 - A.wmax + 1);
    range[1] = lower_bound_lo(A.rec, A.n_inter, r0 + BO);
  }
  __syncthreads();
  const int ta = range[0], tb = range[1];

  double accr[BO], acci[BO];
#pragma unroll
  for (int j = 0; j < BO; ++j) accr[j] = acci[j] = 0.0;

  for (int ts = ta; ts < tb; ts += TT) {
    const int nt = min(TT, tb - ts);
    __syncthreads();
    for (int e = threadIdx.x; e < nt * 16; e += 128) {
      int tt = e >> 4, a = e & 15;
      int row = A.rec[ts + tt].k;
      int g = gi0 + a;
      Ms[tt][a] = g < A.nlf ? A.M[(size_t)row * A.nlf + g] : make_double2(0.0, 0.0);
    }
    for (int e = threadIdx.x; e < nt * 8; e += 128) {
      int tt = e >> 3, a = e & 7;
      int row = A.rec[ts + tt].k;
      int g = gj0 + a;
      M2s[tt][a] = g < A.nlf ? A.M2[(size_t)row * A.nlf + g] : make_double2(0.0, 0.0);
    }
    for (int e = threadIdx.x; e < nt * BO; e += 128) {
      int tt = e / BO, j = e % BO;
      const Trans& t = A.rec[ts + tt];
      int r = r0 + j;
      double w = 0.0;
      if (r < A.nw && r >= t.lo && r <= t.hi) {
        bool in;
        double L = lorentz(A, r, t.e1, t.e2, &in);
        if (in) w = t.c * L;
      }
      Ws[tt][j] = w;
    }
    __syncthreads();
    for (int tt = 0; tt < nt; ++tt) {
      double2 a = Ms[tt][tx], b = M2s[tt][ty];
      double xr = a.x * b.x + a.y * b.y;  // Re(a conj b)
      double xi = a.y * b.x - a.x * b.y;  // Im(a conj b)
#pragma unroll
      for (int j = 0; j < BO; ++j) {
        double w = Ws[tt][j];
        if (w != 0.0) {
          accr[j] = fma(w, xr, accr[j]);
          if (CPLX) acci[j] = fma(w, xi, acci[j]);
        }
      }
    }
  }
  if (gi < A.nlf && gj < A.nlf) {
    const size_t np = (size_t)A.nlf * A.nlf;
    const size_t p = (size_t)gi + (size_t)A.nlf * gj;
#pragma unroll
    for (int j = 0; j < BO; ++j) {
      int r = r0 + j;
      if (r >= A.nw) break;
      if (CPLX) {
        double2* s = reinterpret_cast<double2*>(S) + (size_t)r * np + p;
        double2 v = *s;
        v.x += accr[j];
        v.y += acci[j];
        *s = v;
      } else {
        S[(size_t)r * np + p] += accr[j];
      }
    }
  }
}

int accumulate_fp64(rpa_ctx* c, const Chi0Plan& P, int n_inter, int wmax) {
  if (n_inter == 0) return RPA_OK;
  AccCtx A;
  A.rec = c->d_sorted.as<Trans>();
  A.M = c->d_M.as<double2>();
  const bool two = P.mode == RPA_MODE_CURRENT && (P.pol == RPA_POL_YZ || P.pol == RPA_POL_ZY);
  A.M2 = two ? c->d_M2.as<double2>() : A.M;
  A.nlf = c->nlf;
  A.nw = P.nw;
  A.obase = P.wbase;
  A.wmax = wmax;
  A.n_inter = n_inter;
  A.domega = P.domega;
  A.eta = P.eta;
  A.cut_over_eta = P.cut / P.eta;
  constexpr int BO = 16, TT = 32;
  dim3 grid((P.nw + BO - 1) / BO, (c->nlf + 15) / 16, (c->nlf + 7) / 8);
  if (P.mode == RPA_MODE_CURRENT)
    k_accum_fp64<BO, TT, true><<<grid, 128, 0, c->stream>>>(A, c->d_S.as<double>());
  else
    k_accum_fp64<BO, TT, false><<<grid, 128, 0, c->stream>>>(A, c->d_S.as<double>());
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

// Qeff += c M conj(M2) over the intraband records (sorted tail), one
// (G,G') element per thread, transitions in emission order.
__global__ void k_qeff(const Trans* __restrict__ rec, int t_begin, int t_end, const double2* __restrict__ M,
                       const double2* __restrict__ M2, int nlf, double2* __restrict__ Q) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nlf * nlf) return;
  int gi = p % nlf, gj = p / nlf;
  double qr = 0.0, qi = 0.0;
  for (int t = t_begin; t < t_end; ++t) {
    const Trans& r = rec[t];
    double2 a = M[(size_t)r.k * nlf + gi], b = M2[(size_t)r.k * nlf + gj];
    double xr = a.x * b.x + a.y * b.y, xi = a.y * b.x - a.x * b.y;
    qr = fma(r.c, xr, qr);
    qi = fma(r.c, xi, qi);
  }
  double2 v = Q[p];
  v.x += qr;
  v.y += qi;
  Q[p] = v;
}

int qeff_fp64(rpa_ctx* c, const Chi0Plan& P, int n_inter, int n_trans) {
  if (n_trans <= n_inter) return RPA_OK;
  const bool two = P.pol == RPA_POL_YZ || P.pol == RPA_POL_ZY;
  int np = c->nlf * c->nlf;
  k_qeff<<<(np + 127) / 128, 128, 0, c->stream>>>(c->d_sorted.as<Trans>(), n_inter, n_trans, c->d_M.as<double2>(),
                                                  two ? c->d_M2.as<double2>() : c->d_M.as<double2>(), c->nlf,
                                                  c->d_Q.as<double2>());
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

}  // namespace rpa
