// k_setup.cu -- transition enumeration, Lorentzian windows and their sort.
//
// The reference walks every band pair of every FBZ k-point inside its OpenMP
// loop and tests the occupation cut (Optabs.f90:351-356) or the fixed
// occupied/empty split (Sloss.f90:355-357), then tests the Lorentzian cut for
// each frequency (Sloss.f90:407-411, Optabs.f90:388-399).  Here one block per
// k-point evaluates the same tests once, keeps only pairs whose Lorentzian
// window meets the frequency grid (or the intraband Qeff pairs), and records
// the window [lo, hi] so the accumulation never visits frequencies outside it.
// The window predicate is evaluated in the reference's operation order with
// round-to-nearest intrinsics (no FMA contraction), so window membership is
// identical to a plain IEEE evaluation of the Fortran expression.

#include <cub/cub.cuh>
#include <cmath>
#include <cstring>

#include "rpa_internal.cuh"

namespace rpa {

struct PairCtx {
  const int* kmap;     // 5 per FBZ k: K1,R1,K2,R2,iG0 (0-based)
  const double* E;     // [kibz][nbnd]
  const double2* occ;  // [kibz][nbnd]: (f, Qeff prefactor)
  int nbnd, nocc, mode, nw, obase;
  double domega, eta, cut_over_eta, df_cut, Efermi, tenT, c_charge, c_current;
  int2* scr;           // [ntot][npairs]: (lo | kind << 28, hi) from the count pass
  double half_width;   // eta sqrt(1/cut - 1) / domega: half-width of a window in rows
  double inv_domega;
};

// L(io) >= cut/eta, evaluated as ((o + e1) - e2)^2 + eta^2 without contraction.
__device__ __forceinline__ bool in_window(const PairCtx& P, int r, double e1, double e2) {
  double o = __dmul_rn((double)(r + P.obase), P.domega);
  double dE = __dadd_rn(__dadd_rn(o, e1), -e2);
  double den = __dadd_rn(__dmul_rn(dE, dE), __dmul_rn(P.eta, P.eta));
  double L = __ddiv_rn(P.eta, den);
  return L >= P.cut_over_eta;
}

// Exact window [lo, hi] of rows r in [0, nw), or lo > hi when empty.
__device__ void window_of(const PairCtx& P, double e1, double e2, int* lo_out, int* hi_out) {
  // |dE| <= R with R = eta sqrt(1/cut - 1); centre where o = e2 - e1.  The
  // bracket only has to contain the window (its edges are then found with the
  // exact predicate), so it uses the precomputed half-width and 1/domega.
  double rc = (e2 - e1) * P.inv_domega - (double)P.obase;
  double h = P.half_width;
  double flo = floor(rc - h) - 1.0, fhi = ceil(rc + h) + 1.0;
  if (fhi < 0.0 || flo > (double)(P.nw - 1)) {
    *lo_out = 1;
    *hi_out = 0;
    return;
  }
  int lo = (int)fmax(flo, 0.0), hi = (int)fmin(fhi, (double)(P.nw - 1));
  while (lo <= hi && !in_window(P, lo, e1, e2)) ++lo;
  while (hi >= lo && !in_window(P, hi, e1, e2)) --hi;
  if (lo <= hi) {
    while (lo > 0 && in_window(P, lo - 1, e1, e2)) --lo;
    while (hi < P.nw - 1 && in_window(P, hi + 1, e1, e2)) ++hi;
  }
  *lo_out = lo;
  *hi_out = hi;
}

// Evaluates pair p of k-point ik.  Returns 0 (drop), 1 (interband) or 2 (intraband Qeff).
__device__ int eval_pair(const PairCtx& P, int ik, int p, Trans* t) {
  const int* km = P.kmap + 5 * ik;
  int K1 = km[0], K2 = km[2];
  int n, m;
  if (P.mode == RPA_MODE_CHARGE) {
    int nemp = P.nbnd - P.nocc;
    n = p / nemp;
    m = P.nocc + p % nemp;
  } else {
    n = p / P.nbnd;
    m = p % P.nbnd;
  }
  double e1 = P.E[(size_t)K1 * P.nbnd + n];
  double e2 = P.E[(size_t)K2 * P.nbnd + m];
  t->k = ik;
  t->nm = n | (m << 16);
  t->e1 = e1;
  t->e2 = e2;
  if (P.mode == RPA_MODE_CHARGE) {
    t->c = P.c_charge;
  } else {
    double2 o1 = P.occ[(size_t)K1 * P.nbnd + n];
    double2 o2 = P.occ[(size_t)K2 * P.nbnd + m];
    double df = o1.x - o2.x;
    if (!(fabs(df) >= P.df_cut || n == m)) return 0;
    if (n == m) {
      if (fabs(e1 - P.Efermi) <= P.tenT) {
        t->c = o1.y;
        t->lo = 0;
        t->hi = -1;
        return 2;
      }
      return 0;
    }
    t->c = P.c_current * df;
  }
  int lo, hi;
  window_of(P, e1, e2, &lo, &hi);
  if (lo > hi) return 0;
  t->lo = lo;
  t->hi = hi;
  return 1;
}

// Record of pair p of k-point ik from its kind (1 interband, 2 intraband) and
// window, as eval_pair writes it.
__device__ void fill_pair(const PairCtx& P, int ik, int p, int kind, int lo, int hi, Trans* t) {
  const int* km = P.kmap + 5 * ik;
  const int K1 = km[0], K2 = km[2];
  int n, m;
  if (P.mode == RPA_MODE_CHARGE) {
    const int nemp = P.nbnd - P.nocc;
    n = p / nemp;
    m = P.nocc + p % nemp;
  } else {
    n = p / P.nbnd;
    m = p % P.nbnd;
  }
  t->k = ik;
  t->nm = n | (m << 16);
  t->e1 = P.E[(size_t)K1 * P.nbnd + n];
  t->e2 = P.E[(size_t)K2 * P.nbnd + m];
  if (P.mode == RPA_MODE_CHARGE) {
    t->c = P.c_charge;
  } else {
    const double2 o1 = P.occ[(size_t)K1 * P.nbnd + n];
    t->c = kind == 2 ? o1.y : P.c_current * (o1.x - P.occ[(size_t)K2 * P.nbnd + m].x);
  }
  t->lo = lo;
  t->hi = hi;
}

// The count pass evaluates every pair (the FP64 window search) once and keeps
// its kind and window in P.scr for the emit pass.
__global__ void k_pairs_count(PairCtx P, int k0, int npairs, int* counts, int* maxpairs) {
  int ik = k0 + blockIdx.x;
  int cnt = 0;
  for (int p = threadIdx.x; p < npairs; p += blockDim.x) {
    Trans t;
    const int kind = eval_pair(P, ik, p, &t);
    cnt += kind != 0;
    P.scr[(size_t)ik * npairs + p] = kind ? make_int2(t.lo | (kind << 28), t.hi) : make_int2(0, 0);
  }
  typedef cub::BlockReduce<int, 256> BR;
  __shared__ typename BR::TempStorage tmp;
  int tot = BR(tmp).Sum(cnt);
  if (threadIdx.x == 0) {
    counts[blockIdx.x] = tot;
    atomicMax(maxpairs, tot);
  }
}

// Emits the records of k-point k0+blockIdx.x at offsets[blockIdx.x] in pair
// order (n outer, m inner, as the reference loops), with the sort key.
__global__ void k_pairs_emit(PairCtx P, int k0, int npairs, const long long* offsets, Trans* out,
                             int* keys, int* vals, int key_intra, int* wmax, unsigned long long* winsum) {
  typedef cub::BlockScan<int, 256> BS;
  __shared__ typename BS::TempStorage tmp;
  __shared__ int base;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  long long off = offsets[blockIdx.x];
  int ik = k0 + blockIdx.x;
  int mywmax = 0, myinter = 0;
  unsigned long long mywin = 0;
  for (int p0 = 0; p0 < npairs; p0 += blockDim.x) {
    int p = p0 + threadIdx.x;
    Trans t;
    int kind = 0;
    if (p < npairs) {
      const int2 r = P.scr[(size_t)ik * npairs + p];
      kind = (int)((unsigned)r.x >> 28);
      if (kind) fill_pair(P, ik, p, kind, r.x & 0x0fffffff, r.y, &t);
    }
    int flag = kind != 0, rank, total;
    BS(tmp).ExclusiveSum(flag, rank, total);
    if (flag) {
      long long idx = off + base + rank;
      t.k = blockIdx.x;  // chunk-local k
      out[idx] = t;
      keys[idx] = kind == 1 ? t.lo : key_intra;
      vals[idx] = (int)idx;
      if (kind == 1) {
        mywmax = max(mywmax, t.hi - t.lo + 1);
        ++myinter;
        mywin += (unsigned long long)(t.hi - t.lo + 1);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) base += total;
    __syncthreads();
  }
  if (mywmax) atomicMax(wmax, mywmax);
  if (myinter) atomicAdd(wmax + 2, myinter);
  if (mywin) atomicAdd(winsum, mywin);
}

__global__ void k_gather_sorted(const Trans* in, const int* order, Trans* out, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    int t = order[i];
    Trans r = in[t];
    r.k = t;  // sorted records carry the vertex row index
    out[i] = r;
  }
}

static PairCtx make_pair_ctx(rpa_ctx* c, const Chi0Plan& Pl) {
  PairCtx P;
  P.kmap = c->d_kmap.as<int>();
  P.E = c->d_E.as<double>();
  P.occ = c->d_occ.as<double2>();
  P.nbnd = c->nbnd;
  P.nocc = Pl.nocc;
  P.mode = Pl.mode;
  P.nw = Pl.nw;
  P.obase = Pl.wbase;
  P.domega = Pl.domega;
  P.eta = Pl.eta;
  P.cut_over_eta = Pl.cut / Pl.eta;
  P.df_cut = Pl.df_cut;
  P.Efermi = Pl.Efermi;
  P.tenT = 10.0 * Pl.T;
  P.c_charge = 2.0 / Pl.norm_s;
  P.c_current = -2.0 / Pl.norm_s;
  P.scr = c->d_pairscr.as<int2>();
  const double cut = Pl.cut;
  P.half_width = Pl.eta * std::sqrt(std::fmax(1.0 / cut - 1.0, 0.0)) / Pl.domega;
  P.inv_domega = 1.0 / Pl.domega;
  return P;
}

static int npairs_of(rpa_ctx* c, const Chi0Plan& P) {
  return P.mode == RPA_MODE_CHARGE ? P.nocc * (c->nbnd - P.nocc) : c->nbnd * c->nbnd;
}

// Counts the contributing transitions of every FBZ k-point in [k0, k0+nk)
// into d_counts (host copy returned through counts).
int count_pairs(rpa_ctx* c, const Chi0Plan& Pl, int k0, int nk, std::vector<int>& counts, int* maxp) {
  RPA_TRY(ensure(c, c->d_pairscr, sizeof(int2) * (size_t)(k0 + nk) * npairs_of(c, Pl)));
  PairCtx P = make_pair_ctx(c, Pl);
  RPA_TRY(ensure(c, c->d_counts, sizeof(int) * (size_t)(nk + 1)));
  RPA_TRY(ensure(c, c->d_wmax, 32));
  RPA_CUDA(c, cudaMemsetAsync(c->d_wmax.p, 0, 32, c->stream));
  k_pairs_count<<<nk, 256, 0, c->stream>>>(P, k0, npairs_of(c, Pl), c->d_counts.as<int>(),
                                           c->d_wmax.as<int>() + 1);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  counts.resize(nk);
  RPA_CUDA(c, cudaMemcpyAsync(counts.data(), c->d_counts.p, sizeof(int) * nk, cudaMemcpyDeviceToHost,
                              c->stream));
  int mx = 0;
  RPA_CUDA(c, cudaMemcpyAsync(&mx, c->d_wmax.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  *maxp = mx;
  return RPA_OK;
}

int emit_pairs(rpa_ctx* c, const Chi0Plan& Pl, int k0, int nk, const std::vector<long long>& offsets,
               long long n_trans, int* wmax_out, int* n_inter_out, double* winsum_out) {
  PairCtx P = make_pair_ctx(c, Pl);
  RPA_TRY(ensure(c, c->d_offsets, sizeof(long long) * (size_t)(nk + 1)));
  RPA_TRY(ensure(c, c->d_trans, sizeof(Trans) * (size_t)(n_trans + 1)));
  RPA_TRY(ensure(c, c->d_keys, sizeof(int) * (size_t)(n_trans + 1)));
  RPA_TRY(ensure(c, c->d_vals, sizeof(int) * (size_t)(n_trans + 1)));
  RPA_CUDA(c, cudaMemcpyAsync(c->d_offsets.p, offsets.data(), sizeof(long long) * (nk + 1),
                              cudaMemcpyHostToDevice, c->stream));
  RPA_CUDA(c, cudaMemsetAsync(c->d_wmax.p, 0, 32, c->stream));
  k_pairs_emit<<<nk, 256, 0, c->stream>>>(P, k0, npairs_of(c, Pl), c->d_offsets.as<long long>(),
                                          c->d_trans.as<Trans>(), c->d_keys.as<int>(), c->d_vals.as<int>(),
                                          Pl.nw, c->d_wmax.as<int>(),
                                          reinterpret_cast<unsigned long long*>(c->d_wmax.as<int>() + 4));
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  int w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  RPA_CUDA(c, cudaMemcpyAsync(w, c->d_wmax.p, 32, cudaMemcpyDeviceToHost, c->stream));
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  *wmax_out = w[0];
  *n_inter_out = w[2];
  unsigned long long ws;
  std::memcpy(&ws, w + 4, sizeof ws);
  *winsum_out = (double)ws;
  return RPA_OK;
}

// Stable radix sort of the transitions by window start (intraband records,
// keyed nw, land at the tail in emission order); gathers the sorted records.
int sort_trans(rpa_ctx* c, int n_trans, int nw) {
  if (n_trans == 0) return RPA_OK;
  int end_bit = 1;
  while ((1 << end_bit) <= nw) ++end_bit;
  RPA_TRY(ensure(c, c->d_keys_alt, sizeof(int) * (size_t)n_trans));
  RPA_TRY(ensure(c, c->d_vals_alt, sizeof(int) * (size_t)n_trans));
  size_t tb = 0;
  RPA_CUDA(c, cub::DeviceRadixSort::SortPairs(nullptr, tb, c->d_keys.as<int>(), c->d_keys_alt.as<int>(),
                                              c->d_vals.as<int>(), c->d_vals_alt.as<int>(), n_trans, 0,
                                              end_bit, c->stream));
  RPA_TRY(ensure(c, c->d_cub, tb));
  RPA_CUDA(c, cub::DeviceRadixSort::SortPairs(c->d_cub.p, tb, c->d_keys.as<int>(), c->d_keys_alt.as<int>(),
                                              c->d_vals.as<int>(), c->d_vals_alt.as<int>(), n_trans, 0,
                                              end_bit, c->stream));
  RPA_TRY(ensure(c, c->d_sorted, sizeof(Trans) * ((size_t)n_trans + 64)));  // whole chunks for bulk copies
  k_gather_sorted<<<(n_trans + 255) / 256, 256, 0, c->stream>>>(c->d_trans.as<Trans>(), c->d_vals_alt.as<int>(),
                                                                c->d_sorted.as<Trans>(), n_trans);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}

// ---------------------------------------------------------------------------
// [w][p] (p fastest) -> Fortran (w fastest) for ncomp doubles per element.
template <int NC>
__global__ void k_transpose(const double* __restrict__ src, double* __restrict__ dst, int nw, int np) {
  __shared__ double tile[NC][32][33];
  int p0 = blockIdx.x * 32, w0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int w = w0 + j, p = p0 + threadIdx.x;
    if (w < nw && p < np)
      for (int cc = 0; cc < NC; ++cc) tile[cc][j][threadIdx.x] = src[((size_t)w * np + p) * NC + cc];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int p = p0 + j, w = w0 + threadIdx.x;
    if (w < nw && p < np)
      for (int cc = 0; cc < NC; ++cc) dst[((size_t)p * nw + w) * NC + cc] = tile[cc][threadIdx.x][j];
  }
}

void launch_transpose_wp_to_fortran(const double* src, double* dst, int nw, int np, int ncomp, cudaStream_t s) {
  dim3 grid((np + 31) / 32, (nw + 31) / 32), block(32, 8);
  if (ncomp == 1) k_transpose<1><<<grid, block, 0, s>>>(src, dst, nw, np);
  else k_transpose<2><<<grid, block, 0, s>>>(src, dst, nw, np);
}

}  // namespace rpa
