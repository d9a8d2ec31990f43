// k_dyson.cu -- FP64 local-field Dyson step, one frequency per block.
//
// Reference, per io = 1..no-1 (W/Sloss.f90:452-481):
//   genDielectricEpsilon  eps = I - chi0 V               (Sloss.f90:1210-1234)
//   gjel                  eps <- eps^-1, Gauss-Jordan with full pivoting
//                                                        (W/gjel.f:1-91)
//   genChi                chi = eps^-1 chi0              (Sloss.f90:1236-1253)
//   genWT                 WT  = V + V chi V              (Sloss.f90:1255-1277)
// The pivot search keeps gjel's rule: the candidate set is the rows that are
// not yet pivots and the columns never pivoted, and among equal |a| the last
// one in (row, column) scan order wins (`>= big`).  A repeated pivot column
// is reported as singular (gjel's stop); a zero pivot is counted (gjel prints
// and carries on).  Each block works on its frequency's matrices in a
// per-block global scratch (L1/L2 resident); the stage is FP64-pipe bound,
// and the pivot search (n^2 candidates per step) is most of it: the FP64 path
// ranks candidates by hypot, as gjel's ABS does; the mixed path (MAG2) by
// |a|^2, the same order up to ties that hypot's rounding makes, at a tenth of
// the cost.  The mixed path also forms W as V eps^-1, which equals the
// reference's V + V chi V (see below) with a quarter of its FP64 products.

#include <mutex>

#include "rpa_internal.cuh"

namespace rpa {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// 1/z by Smith's method (no overflow for large |z|).
__device__ __forceinline__ double2 crecip(double2 z) {
  if (fabs(z.x) >= fabs(z.y)) {
    double r = z.y / z.x, d = z.x + z.y * r;
    return make_double2(1.0 / d, -r / d);
  } else {
    double r = z.x / z.y, d = z.x * r + z.y;
    return make_double2(r / d, -1.0 / d);
  }
}

struct DysonArgs {
  const double2* chi0;  // [nwo][n*n] column-major matrices
  const double* V;      // [n*n] column-major
  double2* WT;          // [nwo][n*n]
  double2* epsinv;      // [nwo][n*n] or null
  double2* head;        // [nwo] or null
  double2* scratch;     // [gridDim.x][3][n*n]
  int* flags;           // [0] singular count, [1] zero-pivot count
  int n, nwo;
};

template <bool MAG2>
__global__ void __launch_bounds__(256) k_dyson_fp64(DysonArgs D) {
  extern __shared__ unsigned char smraw[];
  const int n = D.n, nn = n * n;
  int* ipiv = reinterpret_cast<int*>(smraw);
  int* indxr = ipiv + n;
  int* indxc = indxr + n;
  double2* dums = reinterpret_cast<double2*>(smraw + (((size_t)3 * n * sizeof(int) + 15) & ~(size_t)15));
  __shared__ double red_v[256];
  __shared__ int red_e[256];
  __shared__ int sh_bad;

  double2* E = D.scratch + (size_t)blockIdx.x * 3 * nn;
  double2* Cx = E + nn;
  double2* T = Cx + nn;

  for (int io0 = blockIdx.x; io0 < D.nwo; io0 += gridDim.x) {
    const double2* A = D.chi0 + (size_t)io0 * nn;
    // eps = I - A V
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
      int i = e % n, j = e / n;
      double re = (i == j) ? 1.0 : 0.0, im = 0.0;
      for (int k = 0; k < n; ++k) {
        double2 a = A[i + (size_t)n * k];
        double v = D.V[k + (size_t)n * j];
        re -= a.x * v;
        im -= a.y * v;
      }
      E[e] = make_double2(re, im);
    }
    for (int e = threadIdx.x; e < n; e += blockDim.x) ipiv[e] = 0;
    if (threadIdx.x == 0) sh_bad = 0;
    __syncthreads();

    // Gauss-Jordan with full pivoting (gjel)
    int it_done = n;
    for (int it = 0; it < n; ++it) {
      double bv = -1.0;
      int be = -1;
      bool rep = false;
      for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        int j = e / n, k = e % n;  // scan order: row j outer, column k inner
        if (ipiv[j] != 1) {
          int pk = ipiv[k];
          if (pk == 0) {
            double2 a = E[j + (size_t)n * k];
            const double v = MAG2 ? a.x * a.x + a.y * a.y : hypot(a.x, a.y);
            if (v > bv || (v == bv && e > be)) {
              bv = v;
              be = e;
            }
          } else if (pk > 1) {
            rep = true;
          }
        }
      }
      red_v[threadIdx.x] = bv;
      red_e[threadIdx.x] = be;
      if (rep) sh_bad = 1;
      __syncthreads();
      for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
          double v2 = red_v[threadIdx.x + s];
          int e2 = red_e[threadIdx.x + s];
          if (v2 > red_v[threadIdx.x] || (v2 == red_v[threadIdx.x] && e2 > red_e[threadIdx.x])) {
            red_v[threadIdx.x] = v2;
            red_e[threadIdx.x] = e2;
          }
        }
        __syncthreads();
      }
      const int pe = red_e[0];
      if (pe < 0 || sh_bad) {
        if (threadIdx.x == 0) atomicAdd(&D.flags[0], 1);
        it_done = it;
        __syncthreads();
        break;
      }
      const int irow = pe / n, icol = pe % n;
      if (irow != icol) {
        for (int l = threadIdx.x; l < n; l += blockDim.x) {
          double2 t = E[irow + (size_t)n * l];
          E[irow + (size_t)n * l] = E[icol + (size_t)n * l];
          E[icol + (size_t)n * l] = t;
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        ipiv[icol] += 1;
        indxr[it] = irow;
        indxc[it] = icol;
      }
      double2 piv = E[icol + (size_t)n * icol];
      if (threadIdx.x == 0 && piv.x == 0.0 && piv.y == 0.0) atomicAdd(&D.flags[1], 1);
      double2 pinv = crecip(piv);
      __syncthreads();
      for (int l = threadIdx.x; l < n; l += blockDim.x) {
        double2 v = (l == icol) ? make_double2(1.0, 0.0) : E[icol + (size_t)n * l];
        E[icol + (size_t)n * l] = cmul(v, pinv);
      }
      __syncthreads();
      for (int ll = threadIdx.x; ll < n; ll += blockDim.x) dums[ll] = E[ll + (size_t)n * icol];
      __syncthreads();
      for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        int ll = e % n, l = e / n;
        if (ll == icol) continue;
        double2 dum = dums[ll];
        double2 a = (l == icol) ? make_double2(0.0, 0.0) : E[e];
        double2 p = E[icol + (size_t)n * l];
        a.x -= p.x * dum.x - p.y * dum.y;
        a.y -= p.x * dum.y + p.y * dum.x;
        E[e] = a;
      }
      __syncthreads();
    }
    // undo the column interchanges
    for (int l = it_done - 1; l >= 0; --l) {
      int r = indxr[l], cc = indxc[l];
      if (r != cc) {
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
          double2 t = E[k + (size_t)n * r];
          E[k + (size_t)n * r] = E[k + (size_t)n * cc];
          E[k + (size_t)n * cc] = t;
        }
      }
      __syncthreads();
    }
    double2* W = D.WT + (size_t)io0 * nn;
    if constexpr (MAG2) {
      // W = V + V chi V with chi = eps^-1 chi0 and eps = I - chi0 V: since
      // eps^-1 chi0 V = eps^-1 - I, V chi V = V eps^-1 - V and W = V eps^-1,
      // one product and no cancellation between V and V chi V
      for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        const int i = e % n, j = e / n;
        double re = 0.0, im = 0.0;
        for (int k = 0; k < n; ++k) {
          const double v = D.V[i + (size_t)n * k];
          const double2 b = E[k + (size_t)n * j];
          re += v * b.x;
          im += v * b.y;
        }
        W[e] = make_double2(re, im);
        if (D.epsinv) D.epsinv[(size_t)io0 * nn + e] = E[e];
      }
    } else {
      // chi = eps^-1 chi0
      for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        int i = e % n, j = e / n;
        double re = 0.0, im = 0.0;
        for (int k = 0; k < n; ++k) {
          double2 a = E[i + (size_t)n * k], b = A[k + (size_t)n * j];
          re += a.x * b.x - a.y * b.y;
          im += a.x * b.y + a.y * b.x;
        }
        Cx[e] = make_double2(re, im);
      }
      __syncthreads();
      // T = chi V
      for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        int i = e % n, j = e / n;
        double re = 0.0, im = 0.0;
        for (int k = 0; k < n; ++k) {
          double2 a = Cx[i + (size_t)n * k];
          double v = D.V[k + (size_t)n * j];
          re += a.x * v;
          im += a.y * v;
        }
        T[e] = make_double2(re, im);
      }
      __syncthreads();
      // WT = V + V T
      for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        int i = e % n, j = e / n;
        double re = 0.0, im = 0.0;
        for (int k = 0; k < n; ++k) {
          double v = D.V[i + (size_t)n * k];
          double2 b = T[k + (size_t)n * j];
          re += v * b.x;
          im += v * b.y;
        }
        W[e] = make_double2(D.V[e] + re, im);
        if (D.epsinv) D.epsinv[(size_t)io0 * nn + e] = E[e];
      }
    }
    if (D.head && threadIdx.x == 0) D.head[io0] = E[0];
    __syncthreads();
  }
}

static int dyson_grid(rpa_ctx* c, int nwo, int* grid) {
  int dev_sms = 0;
  RPA_CUDA(c, cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, c->device));
  *grid = nwo < 2 * dev_sms ? nwo : 2 * dev_sms;
  return RPA_OK;
}

// Uploads V and sizes every buffer of the Dyson step of the current chi0, so
// that dyson_enqueue allocates nothing.
int dyson_prepare(rpa_ctx* c, const double* V_host, bool want_epsinv) {
  const int n = c->nlf, nn = n * n, nwo = c->last_no - 1;
  RPA_TRY(ensure(c, c->d_V, sizeof(double) * nn));
  RPA_CUDA(c, cudaMemcpyAsync(c->d_V.p, V_host, sizeof(double) * nn, cudaMemcpyHostToDevice, c->stream));
  int grid = 0;
  RPA_TRY(dyson_grid(c, nwo, &grid));
  RPA_TRY(ensure(c, c->d_WT, sizeof(double2) * (size_t)nwo * nn));
  if (want_epsinv) RPA_TRY(ensure(c, c->d_eps, sizeof(double2) * (size_t)nwo * nn));
  RPA_TRY(ensure(c, c->d_tmp, sizeof(double2) * (size_t)grid * 3 * nn + sizeof(double2) * (nwo + 1)));
  RPA_TRY(ensure(c, c->d_flags, sizeof(int) * 4));
  if (c->precision == RPA_PREC_MIXED) RPA_CUDA(c, allow_dynamic_smem(k_dyson_fp64<true>, c->device));
  else RPA_CUDA(c, allow_dynamic_smem(k_dyson_fp64<false>, c->device));
  return RPA_OK;
}

// The Dyson kernel on the context's stream (no allocation, no host wait):
// clears the singular / zero-pivot counters (flags[0..1]; the accumulation's
// status in flags[2..3] is kept) and solves every frequency.
int dyson_enqueue(rpa_ctx* c, bool want_epsinv, const double2** head_dev) {
  const int n = c->nlf, nn = n * n, nwo = c->last_no - 1;
  int grid = 0;
  RPA_TRY(dyson_grid(c, nwo, &grid));
  RPA_CUDA(c, cudaMemsetAsync(c->d_flags.p, 0, sizeof(int) * 2, c->stream));
  DysonArgs D;
  D.chi0 = c->d_chi0.as<double2>();
  D.V = c->d_V.as<double>();
  D.WT = c->d_WT.as<double2>();
  D.epsinv = want_epsinv ? c->d_eps.as<double2>() : nullptr;
  D.scratch = c->d_tmp.as<double2>();
  D.head = D.scratch + (size_t)grid * 3 * nn;
  D.flags = c->d_flags.as<int>();
  D.n = n;
  D.nwo = nwo;
  size_t smem = ((3 * (size_t)n * sizeof(int) + 15) & ~(size_t)15) + sizeof(double2) * n;
  if (c->precision == RPA_PREC_MIXED)
    k_dyson_fp64<true><<<grid, 256, smem, c->stream>>>(D);
  else
    k_dyson_fp64<false><<<grid, 256, smem, c->stream>>>(D);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  if (head_dev) *head_dev = D.head;
  return RPA_OK;
}

int dyson_fp64(rpa_ctx* c, const double* V_host, bool want_epsinv, int* n_singular, int* n_zero,
               const double2** head_dev) {
  RPA_TRY(dyson_prepare(c, V_host, want_epsinv));
  RPA_TRY(dyson_enqueue(c, want_epsinv, head_dev));
  int fl[4];
  RPA_CUDA(c, cudaMemcpyAsync(fl, c->d_flags.p, sizeof(int) * 4, cudaMemcpyDeviceToHost, c->stream));
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  *n_singular = fl[0];
  *n_zero = fl[1];
  return RPA_OK;
}

}  // namespace rpa

namespace rpa {

// ---------------------------------------------------------------------------
// Allocation-free variant of the Dyson step.
//
// Some callers cannot allocate device memory at the point where they need the
// Dyson solve: code running inside a host framework that owns every device
// allocation through its own pool, or latency-critical serving code that must
// not pay for cudaMalloc/cudaFree (an implicit device synchronisation) per
// request.  For them rpa_dyson_noalloc() runs k_dyson_fp64 with its per-block
// workspace in the fixed array below instead of a context-owned buffer.
//
// Limits: n <= NOALLOC_NMAX local fields; the kernel uses at most
// NOALLOC_BLOCKS blocks (one frequency per block at a time), so the array
// holds NOALLOC_BLOCKS * 3 * NOALLOC_NMAX^2 complex doubles = 13.5 MiB, which
// every GPU that loads this library keeps until the process exits.  All calls
// share the array: calls that overlap on the GPU (e.g. on two streams) race.
// The singular/zero-pivot counters at the head of g_noalloc_flags are cleared
// by every call; the workspace itself needs no clearing (each block writes
// every entry it reads).
static constexpr int NOALLOC_NMAX = 96;
static constexpr int NOALLOC_BLOCKS = 32;
static __device__ __align__(256) double2 g_noalloc_scratch[(size_t)NOALLOC_BLOCKS * 3 * NOALLOC_NMAX * NOALLOC_NMAX];
static __device__ __align__(256) int g_noalloc_flags[4];

// Device addresses of the two arrays, looked up once per device with that
// device current (the host-side names are only stand-ins, not device
// addresses).  std::call_once publishes both addresses together, so threads
// making their first calls at the same time see either nothing or both.  The
// addresses belong to the device's primary context: after a cudaDeviceReset
// they are stale, and the entry point must not be used again in the process.
struct NoallocAddrs {
  void* scratch = nullptr;
  void* flags = nullptr;
  int rc = RPA_OK;
};
static NoallocAddrs g_noalloc_addr[64];
static std::once_flag g_noalloc_once[64];

static __global__ void k_noalloc_clear_flags() {
  if (threadIdx.x < 4) g_noalloc_flags[threadIdx.x] = 0;
}

}  // namespace rpa

extern "C" int rpa_dyson_noalloc(const double* chi0, const double* V, int n, int nwo, double* WT, double* head,
                                 void* stream, int* n_singular) {
  using namespace rpa;
  if (!chi0 || !V || !WT || n < 1 || nwo < 1) return RPA_EINVAL;
  if (n > NOALLOC_NMAX) return RPA_EINVAL;  // workspace holds matrices up to NOALLOC_NMAX x NOALLOC_NMAX
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return RPA_ECUDA;
  // One-time set-up on this device: the first call looks up the device
  // addresses of the workspace (loading this library's kernels onto the device
  // if nothing has yet, which reserves the workspace); make that first call
  // before any stream capture.
  std::call_once(g_noalloc_once[dev], [dev]() {
    NoallocAddrs a;
    if (cudaGetSymbolAddress(&a.scratch, g_noalloc_scratch) != cudaSuccess ||
        cudaGetSymbolAddress(&a.flags, g_noalloc_flags) != cudaSuccess)
      a = NoallocAddrs{nullptr, nullptr, RPA_ECUDA};
    g_noalloc_addr[dev] = a;
  });
  const NoallocAddrs& addr = g_noalloc_addr[dev];
  if (addr.rc != RPA_OK) return addr.rc;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int grid = nwo < NOALLOC_BLOCKS ? nwo : NOALLOC_BLOCKS;
  DysonArgs D;
  D.chi0 = reinterpret_cast<const double2*>(chi0);
  D.V = V;
  D.WT = reinterpret_cast<double2*>(WT);
  D.epsinv = nullptr;
  D.head = reinterpret_cast<double2*>(head);
  D.scratch = reinterpret_cast<double2*>(addr.scratch);
  D.flags = reinterpret_cast<int*>(addr.flags);
  D.n = n;
  D.nwo = nwo;
  const size_t smem = ((3 * (size_t)n * sizeof(int) + 15) & ~(size_t)15) + sizeof(double2) * n;
  k_noalloc_clear_flags<<<1, 32, 0, s>>>();
  k_dyson_fp64<false><<<grid, 256, smem, s>>>(D);
  if (cudaGetLastError() != cudaSuccess) return RPA_ECUDA;
  if (n_singular) {
    int fl[2] = {0, 0};
    if (cudaMemcpyAsync(fl, D.flags, sizeof fl, cudaMemcpyDeviceToHost, s) != cudaSuccess) return RPA_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return RPA_ECUDA;
    *n_singular = fl[0];
    if (fl[0]) return RPA_ESINGULAR;
  }
  return RPA_OK;
}

