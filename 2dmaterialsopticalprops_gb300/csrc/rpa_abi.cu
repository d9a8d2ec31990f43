// rpa_abi.cu -- the C ABI (include/rpa_gpu.h) and the host orchestration.
//
// The host side keeps the reference's drivers' contract: arrays arrive in
// their Fortran layouts with 1-based indices, results leave in the same
// layouts.  Everything between (occupations, transition lists, index maps,
// vertices, S0, KK, Dyson) runs on the device of the context.

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>

#include <cuda_fp16.h>

#include "rpa_internal.cuh"

namespace rpa {

// stage implementations (k_*.cu)
int count_pairs(rpa_ctx* c, const Chi0Plan& Pl, int k0, int nk, std::vector<int>& counts, int* maxp);
int emit_pairs(rpa_ctx* c, const Chi0Plan& Pl, int k0, int nk, const std::vector<long long>& offsets,
               long long n_trans, int* wmax_out, int* n_inter_out, double* winsum_out);
int sort_trans(rpa_ctx* c, int n_trans, int nw);
int vertices_fp64(rpa_ctx* c, const Chi0Plan& P, int k0, int nk, int maxpairs, long long n_trans);
int accumulate_fp64(rpa_ctx* c, const Chi0Plan& P, int n_inter, int wmax);
int accumulate_tc(rpa_ctx* c, const Chi0Plan& P, int n_inter, int wmax, const float2* Mf, const float2* Mf2,
                  float amaxM, float amaxM2, double cmax);
int df_to_f64(rpa_ctx* c, size_t n, int nw, bool cplx);
int inverse_perm(rpa_ctx* c, int n, int* pos_of);
int qeff_f32(rpa_ctx* c, int n_inter, int n_trans, const float2* Mf, const float2* Mf2);
int cmax_of(rpa_ctx* c, int n_inter, double* cmax);
int vertices_f32(rpa_ctx* c, const Chi0Plan& P, int k0, int nk, int maxpairs, long long n_trans, const int* pos_of,
                 float2* Mf, float2* Mf2, unsigned* amax);
int vertices_mn(rpa_ctx* c, const Chi0Plan& P, int k0, int nk, long long n_trans, const int* pos_of, float2* Mf,
                float2* Mf2, unsigned* amax, bool* used, int extra_pol);
int qeff_fp64(rpa_ctx* c, const Chi0Plan& P, int n_inter, int n_trans);
int kk_run(rpa_ctx* c, int variant, int no, double domega);
int dyson_fp64(rpa_ctx* c, const double* V_host, bool want_epsinv, int* n_singular, int* n_zero,
               const double2** head_dev);
void kk_matrix(int variant, int no, double domega, std::vector<double>& K, int* nw_out);
int selftest_umma(int which, double* result);
int selftest_wait(double* result);
int selftest_umma_ts(double* result);
int gk_sort_host(const double* k, int npwx, int ngm, const double* g, double ecut, int* ngk, int* igk, double* gk);

static thread_local std::string g_create_err;

int fail(rpa_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  else g_create_err = buf;
  return code;
}

int cuda_fail(rpa_ctx* c, cudaError_t e, const char* what) {
  return fail(c, e == cudaErrorMemoryAllocation ? RPA_ENOMEM : RPA_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

int ensure(rpa_ctx* c, DevBuf& b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (b.bytes >= bytes) return RPA_OK;
  if (b.p) {
    cudaStreamSynchronize(c->stream);
    cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
  }
  cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    b.p = nullptr;
    return fail(c, RPA_ENOMEM, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
  }
  b.bytes = bytes;
  return RPA_OK;
}

void release(DevBuf& b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
}

// ---------------------------------------------------------------------------
__global__ void k_basis_transpose(const double2* __restrict__ src, double2* __restrict__ dst, int nkc, int nbnd,
                                  int npwx) {
  // src [k][b][i] (Fortran C(npwx,nbnd,nks)) -> dst [k][i][b]
  size_t n = (size_t)nkc * nbnd * npwx;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    int b = (int)(e % nbnd);
    size_t r = e / nbnd;
    int i = (int)(r % npwx);
    int k = (int)(r / npwx);
    dst[e] = src[((size_t)k * nbnd + b) * npwx + i];
  }
}

// The same through shared memory, for nbnd <= 64: a block moves a tile of
// BT_I plane waves x all bands of one k-point, reading rows of plane waves and
// writing the tile's contiguous [i][b] run, both coalesced.  The tile row is
// padded by one element so that eight threads reading one column of 16-byte
// elements fall in eight different 16-byte bank groups.
constexpr int BT_I = 64;
__global__ void k_basis_transpose_tiled(const double2* __restrict__ src, double2* __restrict__ dst, int nkc,
                                        int nbnd, int npwx) {
  extern __shared__ double2 bt_tile[];  // [nbnd][BT_I + 1]
  const int nic = (npwx + BT_I - 1) / BT_I;
  for (long long blk = blockIdx.x; blk < (long long)nkc * nic; blk += gridDim.x) {
    const int k = (int)(blk / nic), i0 = (int)(blk % nic) * BT_I;
    const int ni = min(BT_I, npwx - i0);
    const double2* s = src + (size_t)k * nbnd * npwx + i0;
    for (int e = threadIdx.x; e < nbnd * BT_I; e += blockDim.x) {
      const int b = e / BT_I, ii = e - b * BT_I;
      if (ii < ni) bt_tile[b * (BT_I + 1) + ii] = s[(size_t)b * npwx + ii];
    }
    __syncthreads();
    double2* d = dst + ((size_t)k * npwx + i0) * nbnd;
    for (int e = threadIdx.x; e < ni * nbnd; e += blockDim.x) {
      const int ii = e / nbnd, b = e - ii * nbnd;
      d[e] = bt_tile[b * (BT_I + 1) + ii];
    }
    __syncthreads();
  }
}

void launch_basis_transpose(const double2* src, double2* dst, int nkc, int nbnd, int npwx, cudaStream_t s) {
  if (nbnd <= 64) {
    const size_t smem = sizeof(double2) * (size_t)nbnd * (BT_I + 1);
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(k_basis_transpose_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_basis_transpose_tiled<<<4 * 152, 256, smem, s>>>(src, dst, nkc, nbnd, npwx);
  } else {
    k_basis_transpose<<<2048, 256, 0, s>>>(src, dst, nkc, nbnd, npwx);
  }
}

// gidx[k][i] = igk(i, k) - 1 (0-based G index), or i for the legacy basis
__global__ void k_gidx(int* __restrict__ gidx, const int* __restrict__ igk, size_t n, int npwx) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    gidx[e] = igk ? igk[e] - 1 : (int)(e % npwx);
}

__global__ void k_to_f32(const double2* __restrict__ src, float2* __restrict__ dst, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    double2 v = src[e];
    dst[e] = make_float2((float)v.x, (float)v.y);
  }
}

// Coefficients scaled by 2^14 and split into fp16 hi + lo halves (hi = the
// fp16 rounding of 2^14 c, lo = the fp16 rounding of the remainder), stored as
// four planes per plane wave, [re_hi, im_hi, re_lo, im_lo][nbp bands], zero
// beyond nbnd: a run of bands of one plane wave is contiguous for the MN-major
// vertex operands.  Normalised coefficients have |c| <= 1, so 2^14 c stays
// below the fp16 maximum; the representation's absolute resolution is about
// 2^-24 / 2^14 ~ 4e-12 of a coefficient.
__global__ void k_to_planes16(const double2* __restrict__ src, __half* __restrict__ dst, size_t nrows, int nbnd,
                              int nbp) {
  const size_t n = nrows * nbp;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const size_t row = e / nbp;
    const int b = (int)(e % nbp);
    float re = 0.f, im = 0.f;
    if (b < nbnd) {
      const double2 v = src[row * nbnd + b];
      re = (float)v.x * 16384.0f;
      im = (float)v.y * 16384.0f;
    }
    const __half2 hi = __floats2half2_rn(re, im);
    const float2 h = __half22float2(hi);
    const __half2 lo = __floats2half2_rn(re - h.x, im - h.y);
    __half* d = dst + row * 4 * nbp + b;
    d[0] = __low2half(hi);
    d[nbp] = __high2half(hi);
    d[2 * nbp] = __low2half(lo);
    d[3 * nbp] = __high2half(lo);
  }
}

__global__ void k_build_inv(const int* __restrict__ gidx, const int* __restrict__ npw, int* __restrict__ inv,
                            int nks, int npwx, int ng, int* bad) {
  size_t n = (size_t)nks * npwx;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    int k = (int)(e / npwx), i = (int)(e % npwx);
    if (i >= npw[k]) continue;
    int g = gidx[e];
    if (g < 0 || g >= ng) {
      atomicExch(bad, 1);
      continue;
    }
    if (atomicCAS(&inv[(size_t)k * ng + g], -1, i) != -1) atomicExch(bad, 2);
  }
}

static void fill_identity_sym(rpa_ctx* c) {
  c->nsym = 1;
  c->h_R.assign(48 * 9, 0.0);
  for (int i = 0; i < 3; ++i) c->h_R[0 + 48 * (i + 3 * i)] = 1.0;
  c->h_RI = c->h_R;
}

static int upload_symmetry(rpa_ctx* c) {
  // crystal matrices Rc = KC^-1 R KC (row-major [isym][i][j])
  double K[9], Ki[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) K[3 * i + j] = c->KC[i + 3 * j];
  double det = K[0] * (K[4] * K[8] - K[5] * K[7]) - K[1] * (K[3] * K[8] - K[5] * K[6]) + K[2] * (K[3] * K[7] - K[4] * K[6]);
  if (std::fabs(det) < 1e-14) return fail(c, RPA_EINVAL, "reciprocal axes KC are singular");
  Ki[0] = (K[4] * K[8] - K[5] * K[7]) / det;
  Ki[1] = (K[2] * K[7] - K[1] * K[8]) / det;
  Ki[2] = (K[1] * K[5] - K[2] * K[4]) / det;
  Ki[3] = (K[5] * K[6] - K[3] * K[8]) / det;
  Ki[4] = (K[0] * K[8] - K[2] * K[6]) / det;
  Ki[5] = (K[2] * K[3] - K[0] * K[5]) / det;
  Ki[6] = (K[3] * K[7] - K[4] * K[6]) / det;
  Ki[7] = (K[1] * K[6] - K[0] * K[7]) / det;
  Ki[8] = (K[0] * K[4] - K[1] * K[3]) / det;
  c->h_Rc.assign(48 * 9, 0);
  c->h_RIc.assign(48 * 9, 0);
  std::vector<double> Rcart(48 * 9, 0.0);
  for (int s = 0; s < c->nsym; ++s) {
    for (int which = 0; which < 2; ++which) {
      const std::vector<double>& Rf = which ? c->h_RI : c->h_R;
      double R[9], T[9], X[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R[3 * i + j] = Rf[s + 48 * (i + 3 * j)];
      if (!which)
        for (int e = 0; e < 9; ++e) Rcart[9 * s + e] = R[e];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double a = 0;
          for (int k = 0; k < 3; ++k) a += R[3 * i + k] * K[3 * k + j];
          T[3 * i + j] = a;
        }
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double a = 0;
          for (int k = 0; k < 3; ++k) a += Ki[3 * i + k] * T[3 * k + j];
          X[3 * i + j] = a;
        }
      for (int e = 0; e < 9; ++e) {
        double r = std::nearbyint(X[e]);
        if (std::fabs(X[e] - r) > 1e-6)
          return fail(c, RPA_EINVAL, "symmetry %d is not an integer matrix in crystal coordinates", s + 1);
        (which ? c->h_RIc : c->h_Rc)[9 * s + e] = (int)r;
      }
    }
  }
  RPA_TRY(ensure(c, c->d_Rc, sizeof(int) * 48 * 9));
  RPA_TRY(ensure(c, c->d_RIc, sizeof(int) * 48 * 9));
  RPA_TRY(ensure(c, c->d_Rcart, sizeof(double) * 48 * 9));
  RPA_CUDA(c, cudaMemcpy(c->d_Rc.p, c->h_Rc.data(), sizeof(int) * 48 * 9, cudaMemcpyHostToDevice));
  RPA_CUDA(c, cudaMemcpy(c->d_RIc.p, c->h_RIc.data(), sizeof(int) * 48 * 9, cudaMemcpyHostToDevice));
  RPA_CUDA(c, cudaMemcpy(c->d_Rcart.p, Rcart.data(), sizeof(double) * 48 * 9, cudaMemcpyHostToDevice));
  return RPA_OK;
}

// genV, W/Sloss.f90:1173-1208 (q and Glf in 2pi/a0 units, converted with Gcar).
static void genV_host(const rpa_ctx* c, double Gcar, double c0, double eps, std::vector<double>& V) {
  const int n = c->nlf;
  const double pi = 4.0 * std::atan(1.0);
  V.assign((size_t)n * n, 0.0);
  double qx = Gcar * c->q[0], qy = Gcar * c->q[1];
  for (int iG = 0; iG < n; ++iG) {
    const double* gi = &c->h_G[3 * (size_t)c->h_ilf[iG]];
    double gvx = Gcar * gi[0], gvy = Gcar * gi[1], gvz = Gcar * gi[2];
    double Gabs = std::sqrt((qx + gvx) * (qx + gvx) + (qy + gvy) * (qy + gvy));
    if (Gabs == 0.0) Gabs = eps;
    for (int jG = 0; jG < n; ++jG) {
      const double* gj = &c->h_G[3 * (size_t)c->h_ilf[jG]];
      double gjz = Gcar * gj[2];
      double v = 0.0;
      if (gj[0] == gi[0] && gj[1] == gi[1]) {
        v = 4.0 * pi * (1.0 - std::exp(-Gabs * c0)) / (Gabs * c0);
        v = v * (Gabs * Gabs - gvz * gjz);
        v = v / (Gabs * Gabs + gvz * gvz);
        v = v / (Gabs * Gabs + gjz * gjz);
        v = -(double)c->h_parG[iG] * (double)c->h_parG[jG] * v;
        if (gj[2] == gi[2]) v = 4.0 * pi / (Gabs * Gabs + gvz * gvz) + v;
      }
      V[iG + (size_t)n * jG] = v;
    }
  }
}

// V of the current q-point and local fields (genV, Sloss.f90:1173-1208) for
// the batch driver.
void genV_of(const rpa_ctx* c, double c0, double eps, std::vector<double>& V) { genV_host(c, c->last_Gcar, c0, eps, V); }

struct EvTimer {
  rpa_ctx* c;
  int a, b;
  double* out;
};

static double elapsed(rpa_ctx* c, int a, int b) {
  float ms = 0.f;
  cudaEventSynchronize(c->ev[b]);
  cudaEventElapsedTime(&ms, c->ev[a], c->ev[b]);
  return ms;
}

}  // namespace rpa

using namespace rpa;

extern "C" {

int rpa_create(rpa_ctx** out, const rpa_opts* opts) {
  if (!out) return fail(nullptr, RPA_EINVAL, "rpa_create: out is NULL");
  *out = nullptr;
  int dev = opts ? opts->device : 0;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(nullptr, RPA_ECUDA, "rpa_create: no CUDA device (%s)", cudaGetErrorString(e));
  if (dev < 0 || dev >= ndev) return fail(nullptr, RPA_EINVAL, "rpa_create: device %d out of range", dev);
  if (opts && opts->precision != RPA_PREC_FP64 && opts->precision != RPA_PREC_MIXED)
    return fail(nullptr, RPA_EINVAL, "rpa_create: unknown precision %d", opts->precision);
  e = cudaSetDevice(dev);
  if (e != cudaSuccess) return fail(nullptr, RPA_ECUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  rpa_ctx* c = new rpa_ctx();
  c->device = dev;
  c->precision = opts ? opts->precision : RPA_PREC_FP64;
  c->verbose = opts ? opts->verbose : 0;
  c->split_f16 = opts ? opts->split == 0 : true;
  c->tc_seg = (opts && opts->reserved[0] > 0) ? opts->reserved[0] : 1;
  c->vertex_kind = (opts && opts->reserved[1] == 1) ? 1 : 0;
  if (opts && opts->reserved[2] > 0) {
    c->acc_force.gb = opts->reserved[2] & 255;
    c->acc_force.nio = opts->reserved[2] >> 8;
  }
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return fail(nullptr, RPA_ECUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  }
  for (auto& ev : c->ev) cudaEventCreate(&ev);
  fill_identity_sym(c);
  *out = c;
  return RPA_OK;
}

// A context on the parent's device that shares the parent's G list, symmetry
// and basis on the device (no copy) and owns its own k map, q, per-call buffers,
// results and stream, so that several q-points run at once on one resident basis.
int rpa_create_shared(rpa_ctx** out, rpa_ctx* parent, int precision) {
  if (!out || !parent) return fail(nullptr, RPA_EINVAL, "rpa_create_shared: NULL argument");
  *out = nullptr;
  if (parent->parent) return fail(parent, RPA_EINVAL, "rpa_create_shared: parent is itself a shared context");
  if (parent->nks == 0 || parent->ng == 0)
    return fail(parent, RPA_ESTATE, "rpa_create_shared: parent has no G vectors or basis loaded");
  if (precision != -1 && precision != RPA_PREC_FP64 && precision != RPA_PREC_MIXED)
    return fail(parent, RPA_EINVAL, "rpa_create_shared: unknown precision %d", precision);
  if (precision == RPA_PREC_MIXED && parent->precision != RPA_PREC_MIXED)
    return fail(parent, RPA_ESTATE, "rpa_create_shared: the mixed path needs a parent created with RPA_PREC_MIXED");
  cudaError_t e = cudaSetDevice(parent->device);
  if (e != cudaSuccess) return fail(parent, RPA_ECUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  rpa_ctx* c = new rpa_ctx();
  c->device = parent->device;
  c->precision = precision == -1 ? parent->precision : precision;
  c->verbose = parent->verbose;
  c->split_f16 = parent->split_f16;
  c->tc_seg = parent->tc_seg;
  c->vertex_kind = parent->vertex_kind;
  c->vt_table = parent->vt_table;
  c->acc_table = parent->acc_table;
  c->acc_force = parent->acc_force;
  c->nbp = parent->nbp;
  c->ng = parent->ng;
  c->h_miller = parent->h_miller;
  c->h_G = parent->h_G;
  std::memcpy(c->KC, parent->KC, sizeof(c->KC));
  std::memcpy(c->box_lo, parent->box_lo, sizeof(c->box_lo));
  std::memcpy(c->box_dim, parent->box_dim, sizeof(c->box_dim));
  c->nsym = parent->nsym;
  c->h_R = parent->h_R;
  c->h_RI = parent->h_RI;
  c->h_Rc = parent->h_Rc;
  c->h_RIc = parent->h_RIc;
  c->nks = parent->nks;
  c->nbnd = parent->nbnd;
  c->npwx = parent->npwx;
  c->legacy = parent->legacy;
  c->h_npw = parent->h_npw;
  c->h_E = parent->h_E;
  DevBuf* mine[] = {&c->d_miller, &c->d_G, &c->d_box, &c->d_Rc, &c->d_RIc, &c->d_Rcart, &c->d_npw, &c->d_gidx,
                    &c->d_inv, &c->d_coeff, &c->d_coeff32, &c->d_cpl, &c->d_E};
  const DevBuf* theirs[] = {&parent->d_miller, &parent->d_G, &parent->d_box, &parent->d_Rc, &parent->d_RIc,
                            &parent->d_Rcart, &parent->d_npw, &parent->d_gidx, &parent->d_inv, &parent->d_coeff,
                            &parent->d_coeff32, &parent->d_cpl, &parent->d_E};
  for (size_t i = 0; i < sizeof(mine) / sizeof(mine[0]); ++i) *mine[i] = *theirs[i];
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return fail(parent, RPA_ECUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  }
  for (auto& ev : c->ev) cudaEventCreate(&ev);
  c->parent = parent;
  ++parent->children;
  // shared contexts serve requests concurrently: their page-locked staging
  // ring is made now rather than inside the first request
  const int rc = host_io_prepare(c);
  if (rc != RPA_OK) {
    rpa_destroy(c);
    return rc;
  }
  *out = c;
  return RPA_OK;
}

int rpa_destroy(rpa_ctx* c) {
  if (!c) return RPA_OK;
  if (c->children > 0) return fail(c, RPA_ESTATE, "rpa_destroy: %d shared contexts still use this basis", c->children);
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (c->parent) {
    // borrowed from the parent: not ours to free
    DevBuf* borrowed[] = {&c->d_miller, &c->d_G, &c->d_box, &c->d_Rc, &c->d_RIc, &c->d_Rcart, &c->d_npw, &c->d_gidx,
                          &c->d_inv, &c->d_coeff, &c->d_coeff32, &c->d_cpl, &c->d_E};
    for (DevBuf* b : borrowed) *b = DevBuf();
    --c->parent->children;
  }
  DevBuf* bufs[] = {&c->d_miller, &c->d_G, &c->d_box, &c->d_Rc, &c->d_RIc, &c->d_Rcart, &c->d_npw, &c->d_gidx,
                    &c->d_inv, &c->d_coeff, &c->d_coeff32, &c->d_cpl, &c->d_E, &c->d_kmap, &c->d_ktot, &c->d_lf_miller,
                    &c->d_Glf, &c->d_occ, &c->d_counts, &c->d_offsets, &c->d_trans, &c->d_keys, &c->d_keys_alt,
                    &c->d_vals, &c->d_vals_alt, &c->d_sorted, &c->d_M, &c->d_M2, &c->d_Mf, &c->d_Mf2, &c->d_tiles, &c->d_tilesA, &c->d_gmap, &c->d_ginv, &c->d_vbt, &c->d_ybt, &c->d_ptab, &c->d_order, &c->d_cub, &c->d_wmax, &c->d_pairscr,
                    &c->d_ntrans, &c->d_S, &c->d_Sdf, &c->d_Q, &c->d_chi0, &c->d_kk[0], &c->d_kk[1], &c->d_kkf[0], &c->d_kkf[1], &c->d_kkw, &c->d_V, &c->d_eps, &c->d_WT,
                    &c->d_flags, &c->d_tmp};
  for (DevBuf* b : bufs) release(*b);
  host_io_release(c);
  for (auto& ev : c->ev)
    if (ev) cudaEventDestroy(ev);
  cudaStreamDestroy(c->stream);
  delete c;
  return RPA_OK;
}

const char* rpa_last_error(const rpa_ctx* c) { return c ? c->err.c_str() : g_create_err.c_str(); }

int rpa_set_gvectors(rpa_ctx* c, int ng, const int* miller, const double* G, const double* KC) {
  if (c) c->gmap_valid = c->ginv_valid = c->vstash.valid = false;
  if (c && (c->parent || c->children > 0))
    return fail(c, RPA_ESTATE, "rpa_set_gvectors: the G list and basis are shared between contexts");
  if (!c || ng <= 0 || !miller || !G || !KC) return fail(c, RPA_EINVAL, "rpa_set_gvectors: bad arguments");
  cudaSetDevice(c->device);
  if (miller[0] != 0 || miller[1] != 0 || miller[2] != 0)
    return fail(c, RPA_EINVAL, "G(1) is not (0,0,0)");
  c->ng = ng;
  c->h_miller.assign(miller, miller + 3 * (size_t)ng);
  c->h_G.assign(G, G + 3 * (size_t)ng);
  std::memcpy(c->KC, KC, sizeof(double) * 9);
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int g = 0; g < ng; ++g)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], miller[3 * g + d]);
      hi[d] = std::max(hi[d], miller[3 * g + d]);
    }
  size_t vol = 1;
  for (int d = 0; d < 3; ++d) {
    c->box_lo[d] = lo[d];
    c->box_dim[d] = hi[d] - lo[d] + 1;
    vol *= (size_t)c->box_dim[d];
  }
  if (vol > ((size_t)1 << 31)) return fail(c, RPA_EINVAL, "Miller index range too large");
  std::vector<int> box(vol, -1);
  for (int g = 0; g < ng; ++g) {
    size_t idx = ((size_t)(miller[3 * g] - lo[0]) * c->box_dim[1] + (miller[3 * g + 1] - lo[1])) * c->box_dim[2] +
                 (miller[3 * g + 2] - lo[2]);
    if (box[idx] >= 0) return fail(c, RPA_EINVAL, "G vector %d repeats G vector %d", g + 1, box[idx] + 1);
    box[idx] = g;
  }
  RPA_TRY(ensure(c, c->d_miller, sizeof(int) * 3 * (size_t)ng));
  RPA_TRY(ensure(c, c->d_G, sizeof(double) * 3 * (size_t)ng));
  RPA_TRY(ensure(c, c->d_box, sizeof(int) * vol));
  RPA_CUDA(c, cudaMemcpy(c->d_miller.p, miller, sizeof(int) * 3 * (size_t)ng, cudaMemcpyHostToDevice));
  RPA_CUDA(c, cudaMemcpy(c->d_G.p, G, sizeof(double) * 3 * (size_t)ng, cudaMemcpyHostToDevice));
  RPA_CUDA(c, cudaMemcpy(c->d_box.p, box.data(), sizeof(int) * vol, cudaMemcpyHostToDevice));
  return upload_symmetry(c);
}

int rpa_set_symmetry(rpa_ctx* c, int nsym, const double* R, const double* RI) {
  if (c) c->gmap_valid = c->ginv_valid = c->vstash.valid = false;
  if (c && (c->parent || c->children > 0))
    return fail(c, RPA_ESTATE, "rpa_set_symmetry: the G list and basis are shared between contexts");
  if (!c || nsym < 1 || nsym > 48 || !R || !RI) return fail(c, RPA_EINVAL, "rpa_set_symmetry: bad arguments");
  if (c->ng == 0) return fail(c, RPA_ESTATE, "rpa_set_symmetry: call rpa_set_gvectors first");
  cudaSetDevice(c->device);
  c->nsym = nsym;
  c->h_R.assign(R, R + 48 * 9);
  c->h_RI.assign(RI, RI + 48 * 9);
  return upload_symmetry(c);
}

int rpa_load_basis(rpa_ctx* c, int nks, int nbnd, int npwx, const int* npw, const int* igk, const double* coeff,
                   const double* E) {
  if (c && (c->parent || c->children > 0))
    return fail(c, RPA_ESTATE, "rpa_load_basis: the G list and basis are shared between contexts");
  if (c) c->gmap_valid = c->ginv_valid = c->vstash.valid = false;
  if (!c || nks <= 0 || nbnd <= 0 || npwx <= 0 || !npw || !coeff || !E)
    return fail(c, RPA_EINVAL, "rpa_load_basis: bad arguments");
  if (c->ng == 0) return fail(c, RPA_ESTATE, "rpa_load_basis: call rpa_set_gvectors first");
  if (nbnd > 4096) return fail(c, RPA_EINVAL, "rpa_load_basis: nbnd too large");
  cudaSetDevice(c->device);
  for (int k = 0; k < nks; ++k)
    if (npw[k] < 1 || npw[k] > npwx) return fail(c, RPA_EINVAL, "npw(%d) = %d outside 1..npwx", k + 1, npw[k]);
  c->nks = nks;
  c->nbnd = nbnd;
  c->npwx = npwx;
  c->legacy = igk == nullptr;
  c->h_npw.assign(npw, npw + nks);
  if (c->legacy) {
    for (int k = 0; k < nks; ++k)
      if (npw[k] > c->ng) return fail(c, RPA_EINVAL, "npw(%d) exceeds NG in legacy mode", k + 1);
  }
  c->h_E.resize((size_t)nks * nbnd);
  for (int k = 0; k < nks; ++k)
    for (int b = 0; b < nbnd; ++b) c->h_E[(size_t)k * nbnd + b] = E[k + (size_t)nks * b];
  cudaEventRecord(c->ev[6], c->stream);
  RPA_TRY(ensure(c, c->d_npw, sizeof(int) * nks));
  RPA_TRY(ensure(c, c->d_E, sizeof(double) * (size_t)nks * nbnd));
  RPA_TRY(ensure(c, c->d_gidx, sizeof(int) * (size_t)nks * npwx));
  RPA_CUDA(c, cudaMemcpyAsync(c->d_npw.p, npw, sizeof(int) * nks, cudaMemcpyHostToDevice, c->stream));
  RPA_CUDA(c, cudaMemcpyAsync(c->d_E.p, c->h_E.data(), sizeof(double) * (size_t)nks * nbnd, cudaMemcpyHostToDevice,
                              c->stream));
  if (igk)
    RPA_CUDA(c, cudaMemcpyAsync(c->d_gidx.p, igk, sizeof(int) * (size_t)nks * npwx, cudaMemcpyHostToDevice, c->stream));
  k_gidx<<<1024, 256, 0, c->stream>>>(c->d_gidx.as<int>(), igk ? c->d_gidx.as<int>() : nullptr, (size_t)nks * npwx,
                                      npwx);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  if (!c->legacy) {
    RPA_TRY(ensure(c, c->d_inv, sizeof(int) * (size_t)nks * c->ng));
    RPA_TRY(ensure(c, c->d_flags, sizeof(int) * 4));
    RPA_CUDA(c, cudaMemsetAsync(c->d_inv.p, 0xff, sizeof(int) * (size_t)nks * c->ng, c->stream));
    RPA_CUDA(c, cudaMemsetAsync(c->d_flags.p, 0, sizeof(int) * 4, c->stream));
    k_build_inv<<<1024, 256, 0, c->stream>>>(c->d_gidx.as<int>(), c->d_npw.as<int>(), c->d_inv.as<int>(), nks, npwx,
                                             c->ng, c->d_flags.as<int>());
    RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
    int bad = 0;
    RPA_CUDA(c, cudaMemcpyAsync(&bad, c->d_flags.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    RPA_CUDA(c, cudaStreamSynchronize(c->stream));
    if (bad == 1) return fail(c, RPA_EINVAL, "igk entry outside 1..NG");
    if (bad == 2) return fail(c, RPA_EINVAL, "igk repeats a G vector within one k-point");
  }
  // coefficients: raw Fortran blocks, transposed to [k][i][b] on the device
  const size_t per_k = (size_t)nbnd * npwx;
  RPA_TRY(ensure(c, c->d_coeff, sizeof(double2) * per_k * nks));
  RPA_TRY(upload_basis(c, coeff, nks, nbnd, npwx, c->d_coeff.as<double2>()));
  if (c->precision == RPA_PREC_MIXED) {
    // the tensor-core vertex kernel keeps plane-wave positions in int16 maps and
    // band pairs in an int16 table; larger bases need the FP32 CUDA-core vertex
    // kernel, which the caller must choose (opts.reserved[1] = 1)
    if (c->vertex_kind == 0 && (npwx > 32767 || nbnd > 181))
      return fail(c, RPA_EINVAL,
                  "rpa_load_basis: the mixed path's tensor-core vertices take at most 32767 plane waves and 181 "
                  "bands per k-point (npwx=%d, nbnd=%d); create the context with opts.reserved[1] = 1 for the "
                  "FP32 CUDA-core vertex kernel, or use RPA_PREC_FP64", npwx, nbnd);
    // the FP32 copy feeds the CUDA-core vertex kernel only
    if (c->vertex_kind == 1) {
      RPA_TRY(ensure(c, c->d_coeff32, sizeof(float2) * per_k * nks));
      k_to_f32<<<2048, 256, 0, c->stream>>>(c->d_coeff.as<double2>(), c->d_coeff32.as<float2>(), per_k * nks);
      RPA_CUDA(c, cudaGetLastError());
      ++c->launches;
    } else {
      release(c->d_coeff32);
    }
    c->nbp = (nbnd + 7) / 8 * 8;
    RPA_TRY(ensure(c, c->d_cpl, sizeof(__half) * (size_t)nks * npwx * 4 * c->nbp));
    k_to_planes16<<<2048, 256, 0, c->stream>>>(c->d_coeff.as<double2>(), c->d_cpl.as<__half>(), (size_t)nks * npwx,
                                               nbnd, c->nbp);
    RPA_CUDA(c, cudaGetLastError());
    ++c->launches;
  }
  cudaEventRecord(c->ev[7], c->stream);
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  c->stage_ms[5] = elapsed(c, 6, 7);
  c->have_S = c->have_chi0 = c->have_W = false;
  return RPA_OK;
}

int rpa_kmap(rpa_ctx* c, int ntot, const double* ktot, const int* K1, const int* R1, const int* K2, const int* R2,
             const int* iG0) {
  if (c) c->gmap_valid = c->ginv_valid = c->vstash.valid = false;
  if (!c || ntot <= 0 || !ktot || !K1 || !R1 || !K2 || !R2 || !iG0)
    return fail(c, RPA_EINVAL, "rpa_kmap: bad arguments");
  if (c->nks == 0) return fail(c, RPA_ESTATE, "rpa_kmap: call rpa_load_basis first");
  cudaSetDevice(c->device);
  std::vector<int> km(5 * (size_t)ntot);
  for (int k = 0; k < ntot; ++k) {
    int v[5] = {K1[k] - 1, R1[k] - 1, K2[k] - 1, R2[k] - 1, iG0[k] - 1};
    if (v[0] < 0 || v[0] >= c->nks || v[2] < 0 || v[2] >= c->nks)
      return fail(c, RPA_EINVAL, "K1/K2 of k-point %d outside 1..nks", k + 1);
    if (v[1] < 0 || v[1] >= c->nsym || v[3] < 0 || v[3] >= c->nsym)
      return fail(c, RPA_EINVAL, "R1/R2 of k-point %d outside 1..Nsym", k + 1);
    if (v[4] < 0 || v[4] >= c->ng) return fail(c, RPA_EINVAL, "iG0 of k-point %d outside 1..NG", k + 1);
    for (int j = 0; j < 5; ++j) km[5 * (size_t)k + j] = v[j];
  }
  c->ntot = ntot;
  c->h_kmap.swap(km);
  c->h_ktot.assign(ktot, ktot + 3 * (size_t)ntot);
  RPA_TRY(ensure(c, c->d_kmap, sizeof(int) * 5 * (size_t)ntot));
  RPA_TRY(ensure(c, c->d_ktot, sizeof(double) * 3 * (size_t)ntot));
  RPA_CUDA(c, cudaMemcpy(c->d_kmap.p, c->h_kmap.data(), sizeof(int) * 5 * (size_t)ntot, cudaMemcpyHostToDevice));
  RPA_CUDA(c, cudaMemcpy(c->d_ktot.p, ktot, sizeof(double) * 3 * (size_t)ntot, cudaMemcpyHostToDevice));
  c->have_S = c->have_chi0 = c->have_W = false;
  return RPA_OK;
}

int rpa_set_q(rpa_ctx* c, const double* q, int nlf, const int* ilf, const int* parG) {
  if (c) c->gmap_valid = c->ginv_valid = c->vstash.valid = false;
  if (!c || !q || nlf <= 0 || !ilf) return fail(c, RPA_EINVAL, "rpa_set_q: bad arguments");
  if (nlf > 1000) return fail(c, RPA_EINVAL, "Nlf = %d exceeds the gjel limit NMAX = 1000", nlf);
  if (c->ng == 0) return fail(c, RPA_ESTATE, "rpa_set_q: call rpa_set_gvectors first");
  cudaSetDevice(c->device);
  std::vector<int> lm(3 * (size_t)nlf), il(nlf), pg(nlf, 1);
  std::vector<double> gl(3 * (size_t)nlf);
  for (int i = 0; i < nlf; ++i) {
    int g = ilf[i] - 1;
    if (g < 0 || g >= c->ng) return fail(c, RPA_EINVAL, "ilf(%d) outside 1..NG", i + 1);
    il[i] = g;
    for (int d = 0; d < 3; ++d) {
      lm[3 * i + d] = c->h_miller[3 * (size_t)g + d];
      gl[3 * i + d] = c->h_G[3 * (size_t)g + d];
    }
    if (parG) {
      if (parG[i] != 1 && parG[i] != -1) return fail(c, RPA_EINVAL, "parG(%d) must be +1 or -1", i + 1);
      pg[i] = parG[i];
    }
  }
  c->h_ilf.swap(il);
  c->h_parG.swap(pg);
  for (int d = 0; d < 3; ++d) c->q[d] = q[d];
  c->nlf = nlf;
  RPA_TRY(ensure(c, c->d_lf_miller, sizeof(int) * 3 * (size_t)nlf));
  RPA_TRY(ensure(c, c->d_Glf, sizeof(double) * 3 * (size_t)nlf));
  RPA_CUDA(c, cudaMemcpy(c->d_lf_miller.p, lm.data(), sizeof(int) * lm.size(), cudaMemcpyHostToDevice));
  RPA_CUDA(c, cudaMemcpy(c->d_Glf.p, gl.data(), sizeof(double) * gl.size(), cudaMemcpyHostToDevice));
  c->have_q = true;
  c->have_S = c->have_chi0 = c->have_W = false;
  return RPA_OK;
}

// every argument but the polarisation equal (the transitions and their order
// depend on these alone)
static bool same_chi0_args(const rpa_chi0_args& x, const rpa_chi0_args& y) {
  return x.mode == y.mode && x.ngd == y.ngd && x.nocc == y.nocc && x.no == y.no && x.ntot_norm == y.ntot_norm &&
         x.domega == y.domega && x.eta == y.eta && x.lor_cut == y.lor_cut && x.df_cut == y.df_cut && x.T == y.T &&
         x.Efermi == y.Efermi && x.Vcell == y.Vcell && x.Gcar == y.Gcar;
}

int rpa_chi0_prefetch(rpa_ctx* c, int pol) {
  if (!c) return fail(c, RPA_EINVAL, "rpa_chi0_prefetch: bad arguments");
  if (pol != -1 && pol != RPA_POL_XX && pol != RPA_POL_YY && pol != RPA_POL_ZZ)
    return fail(c, RPA_EINVAL, "rpa_chi0_prefetch: pol must be RPA_POL_XX, YY, ZZ or -1");
  c->prefetch_pol = pol;
  return RPA_OK;
}

int rpa_chi0(rpa_ctx* c, const rpa_chi0_args* a, double* S0_out, double* Qeff_out) {
  if (!c || !a) return fail(c, RPA_EINVAL, "rpa_chi0: bad arguments");
  if (c->nks == 0 || c->ntot == 0 || !c->have_q)
    return fail(c, RPA_ESTATE, "rpa_chi0: basis, k map and q must be set first");
  if (a->mode != RPA_MODE_CHARGE && a->mode != RPA_MODE_CURRENT)
    return fail(c, RPA_EINVAL, "rpa_chi0: unknown mode %d", a->mode);
  if (a->pol < RPA_POL_XX || a->pol > RPA_POL_ZY) return fail(c, RPA_EINVAL, "rpa_chi0: unknown pol %d", a->pol);
  if (a->no < 3) return fail(c, RPA_EINVAL, "rpa_chi0: no must be >= 3");
  if (!(a->domega > 0) || !(a->eta > 0) || !(a->Vcell > 0)) return fail(c, RPA_EINVAL, "rpa_chi0: domega, eta, Vcell must be > 0");
  if (a->mode == RPA_MODE_CHARGE && (a->nocc < 1 || a->nocc >= c->nbnd))
    return fail(c, RPA_EINVAL, "rpa_chi0: nocc must be in 1..nbnd-1");
  if (a->mode == RPA_MODE_CURRENT && !(a->T > 0)) return fail(c, RPA_EINVAL, "rpa_chi0: T must be > 0");
  cudaSetDevice(c->device);
  if (!c->vt_forced) {
    // tuned vertex configuration of this shape, if any
    const auto it = c->vt_table.find(vtx_tune_key(a->mode, c->nbnd, a->mode == RPA_MODE_CHARGE ? a->nocc : 0, c->nlf));
    c->vt_cur = it != c->vt_table.end() ? it->second : rpa_ctx::VtxTune();
  }

  Chi0Plan P;
  P.mode = a->mode;
  P.pol = a->pol;
  P.no = a->no;
  P.nw = a->mode == RPA_MODE_CHARGE ? a->no : 2 * a->no + 1;
  P.wbase = a->mode == RPA_MODE_CHARGE ? 0 : -a->no;
  P.nocc = a->nocc;
  P.domega = a->domega;
  P.eta = a->eta;
  P.cut = a->mode == RPA_MODE_CHARGE ? 1.0e-3 : a->lor_cut;
  P.df_cut = a->df_cut;
  P.T = a->T;
  P.Efermi = a->Efermi;
  P.Gcar = a->Gcar;
  P.ntot_norm = a->ntot_norm > 0 ? a->ntot_norm : c->ntot;
  const double pi = 4.0 * std::atan(1.0);
  P.norm_s = pi * P.ntot_norm * a->Vcell;
  P.norm_q = P.ntot_norm * a->Vcell;
  P.nsum_legacy = 0;
  if (c->legacy) {
    if (a->ngd < 1) return fail(c, RPA_EINVAL, "rpa_chi0: NGd must be >= 1 without an igk map");
    for (int k = 0; k < c->ntot; ++k) {
      int K1 = c->h_kmap[5 * k], K2 = c->h_kmap[5 * k + 2];
      if (a->ngd > c->h_npw[K1]) return fail(c, RPA_EINVAL, "NGd is bigger than NG1=%d", c->h_npw[K1]);
      if (a->ngd > c->h_npw[K2]) return fail(c, RPA_EINVAL, "NGd is bigger than NG2=%d", c->h_npw[K2]);
    }
    P.nsum_legacy = a->ngd;
  }

  // occupations (genOccupation, Optabs.f90:935-951) and Qeff prefactors on the host
  {
    std::vector<double> occ(2 * (size_t)c->nks * c->nbnd, 0.0);
    if (a->mode == RPA_MODE_CURRENT) {
      for (size_t i = 0; i < (size_t)c->nks * c->nbnd; ++i) {
        double x = (c->h_E[i] - a->Efermi) / a->T, expo, f;
        if (x < -20) {
          expo = 0.0;
          f = 1.0;
        } else if (x > 20) {
          expo = x;
          f = 0.0;
        } else {
          expo = std::exp(x);
          f = 1.0 / (expo + 1.0);
        }
        double fact = expo / ((expo + 1.0) * (expo + 1.0));
        fact = -fact / a->T;
        occ[2 * i] = f;
        occ[2 * i + 1] = 2.0 * fact / P.norm_q;
      }
    }
    RPA_TRY(ensure(c, c->d_occ, sizeof(double) * occ.size()));
    RPA_CUDA(c, cudaMemcpyAsync(c->d_occ.p, occ.data(), sizeof(double) * occ.size(), cudaMemcpyHostToDevice, c->stream));
  }
  const int np = c->nlf * c->nlf;
  const bool cplx = a->mode == RPA_MODE_CURRENT;
  const size_t s_bytes = (size_t)P.nw * np * (cplx ? 16 : 8);
  RPA_TRY(ensure(c, c->d_S, s_bytes));
  c->s_sym = false;
  c->acc_last_gb = c->acc_last_nio = 0;
  c->deferred = false;
  if (c->defer_acc && c->precision != RPA_PREC_MIXED)
    return fail(c, RPA_EINVAL, "rpa_chi0: a deferred accumulation needs the mixed path");
  RPA_TRY(ensure(c, c->d_Q, sizeof(double2) * np));
  RPA_CUDA(c, cudaMemsetAsync(c->d_S.p, 0, s_bytes, c->stream));
  if (c->precision == RPA_PREC_MIXED) {
    RPA_TRY(ensure(c, c->d_Sdf, s_bytes));  // one (hi, lo) float pair per double of S0
    RPA_CUDA(c, cudaMemsetAsync(c->d_Sdf.p, 0, s_bytes, c->stream));
  }
  RPA_CUDA(c, cudaMemsetAsync(c->d_Q.p, 0, sizeof(double2) * np, c->stream));

  RPA_TRY(ensure(c, c->d_flags, sizeof(int) * 4));
  RPA_CUDA(c, cudaMemsetAsync(c->d_flags.p, 0, sizeof(int) * 4, c->stream));
  double t_pairs = 0, t_vert = 0, t_acc = 0;
  double st_trans = 0, st_win = 0, st_mac = 0, st_launch = 0;
  std::vector<int> counts;
  int maxp = 0;
  cudaEventRecord(c->ev[0], c->stream);
  const bool two = cplx && (a->pol == RPA_POL_YZ || a->pol == RPA_POL_ZY);
  // vertices of this polarisation computed beside the previous call
  // (rpa_chi0_prefetch): that call's transitions, their window-sorted records
  // and its vertex rows for this polarisation are still on the device (the
  // same arguments, k map, q and basis give the same transitions)
  bool from_stash = c->vstash.valid && c->precision == RPA_PREC_MIXED && cplx && !two &&
                    c->vstash.pol == a->pol && same_chi0_args(c->vstash.args, *a);
  c->vstash.valid = false;
  if (from_stash) {
    counts = c->vstash.counts;
    maxp = c->vstash.maxp;
  } else {
    RPA_TRY(count_pairs(c, P, 0, c->ntot, counts, &maxp));
  }
  const int extra_pol = c->precision == RPA_PREC_MIXED && cplx && !two && c->vertex_kind != 1 &&
                                c->prefetch_pol >= 0 && c->prefetch_pol != a->pol
                            ? c->prefetch_pol
                            : -1;
  c->prefetch_pol = -1;
  // per-transition device memory: FP64 vertices (FP64 path) or FP32 vertex rows
  // plus pre-split tiles (mixed path), records, keys and sort buffers
  const size_t per_trans =
      (c->precision == RPA_PREC_MIXED
           ? (size_t)c->nlf * sizeof(float2) * (two || extra_pol >= 0 ? 2 : 1) + (cplx ? 4 : 2) * 96 * 128 / 32 *
                                                                    (size_t)((c->nlf + 95) / 96)
           : (size_t)c->nlf * sizeof(double2) * (two ? 2 : 1)) +
      2 * sizeof(Trans) + 24;
  size_t free_b = 0, total_b = 0;
  RPA_CUDA(c, cudaMemGetInfo(&free_b, &total_b));
  const size_t budget = std::max<size_t>((size_t)1 << 30, std::min<size_t>(free_b / 2, (size_t)96 << 30));
  size_t max_trans = std::max<size_t>(budget / per_trans, (size_t)maxp + 1);
  max_trans = std::min<size_t>(max_trans, (size_t)1 << 30);
  if (from_stash) {
    long long all = 0;
    for (int k = 0; k < c->ntot; ++k) all += counts[k];
    if (all != c->vstash.tot || (size_t)all > max_trans) {
      // not one chunk any more: count again (the pair scratch is rebuilt too)
      from_stash = false;
      RPA_TRY(count_pairs(c, P, 0, c->ntot, counts, &maxp));
    }
  }
  int k0 = 0;
  bool stashed = false;
  while (k0 < c->ntot) {
    long long tot = 0;
    int k1 = k0;
    while (k1 < c->ntot && (size_t)(tot + counts[k1]) <= max_trans) tot += counts[k1++];
    if (k1 == k0) return fail(c, RPA_EINVAL, "rpa_chi0: one k-point exceeds the transition budget");
    if (c->defer_acc && (k0 > 0 || k1 < c->ntot))
      return fail(c, RPA_EINVAL, "rpa_chi0: a deferred accumulation needs the transitions of all k-points in one chunk");
    int nk = k1 - k0;
    std::vector<long long> off(nk + 1, 0);
    for (int i = 0; i < nk; ++i) off[i + 1] = off[i] + counts[k0 + i];
    int wmax = 0, n_inter = 0;
    double winsum = 0;
    cudaEventRecord(c->ev[1], c->stream);
    if (from_stash) {
      n_inter = c->vstash.n_inter;
      wmax = c->vstash.wmax;
      winsum = c->vstash.winsum;
    } else {
      RPA_TRY(emit_pairs(c, P, k0, nk, off, tot, &wmax, &n_inter, &winsum));
      RPA_TRY(sort_trans(c, (int)tot, P.nw));
    }
    if (c->precision == RPA_PREC_MIXED) {
      // FP32 vertices written straight into the window-sorted rows (the
      // transitions and their sorted order are those of the previous call when
      // its stashed rows are used: same arguments, k map, q and basis)
      const bool whole = k0 == 0 && k1 == c->ntot;
      const bool use_stash = from_stash && whole;
      const int xpol = whole ? extra_pol : -1;
      const size_t mrows = ((size_t)tot + 31) / 32 * 32 + 32;
      if (use_stash) std::swap(c->d_Mf, c->d_Mf2);
      RPA_TRY(ensure(c, c->d_Mf, sizeof(float2) * mrows * c->nlf));
      if (two || xpol >= 0) RPA_TRY(ensure(c, c->d_Mf2, sizeof(float2) * mrows * c->nlf));
      RPA_TRY(ensure(c, c->d_counts, sizeof(int) * ((size_t)tot + 1 > (size_t)c->ntot + 1 ? (size_t)tot + 1
                                                                                            : (size_t)c->ntot + 1)));
      float2* Mf = c->d_Mf.as<float2>();
      float2* Mf2 = two ? c->d_Mf2.as<float2>() : Mf;
      float2* Mx = xpol >= 0 ? c->d_Mf2.as<float2>() : Mf2;  // second vertex set of the pass
      const size_t pad0 = (size_t)tot * c->nlf, pad1 = mrows * c->nlf;
      RPA_CUDA(c, cudaMemsetAsync(Mf + pad0, 0, sizeof(float2) * (pad1 - pad0), c->stream));
      if (two || xpol >= 0) RPA_CUDA(c, cudaMemsetAsync(Mx + pad0, 0, sizeof(float2) * (pad1 - pad0), c->stream));
      int* pos_of = c->d_counts.as<int>();
      if (!use_stash) RPA_TRY(inverse_perm(c, (int)tot, pos_of));
      RPA_TRY(ensure(c, c->d_ntrans, 32));
      RPA_CUDA(c, cudaMemsetAsync(c->d_ntrans.p, 0, 32, c->stream));
      cudaEventRecord(c->ev[2], c->stream);
      if (use_stash) {
        // nothing to compute: the rows are in d_Mf
      } else if (c->vertex_kind == 1) {
        RPA_TRY(vertices_f32(c, P, k0, nk, maxp, tot, pos_of, Mf, Mf2, c->d_ntrans.as<unsigned>()));
      } else {
        bool used_tc = false;
        RPA_TRY(vertices_mn(c, P, k0, nk, tot, pos_of, Mf, two ? Mf2 : Mx, c->d_ntrans.as<unsigned>(), &used_tc,
                            xpol));
        if (!used_tc && tot > 0) return fail(c, RPA_ESTATE, "rpa_chi0: the tensor-core vertex kernel did not run");
      }
      cudaEventRecord(c->ev[3], c->stream);
      double cmax = 0.0;
      RPA_TRY(cmax_of(c, n_inter, &cmax));
      unsigned am[2] = {0, 0};
      RPA_CUDA(c, cudaMemcpy(am, c->d_ntrans.p, 8, cudaMemcpyDeviceToHost));
      float amM, amM2;
      std::memcpy(&amM, &am[0], 4);
      std::memcpy(&amM2, &am[1], 4);
      if (use_stash) amM = c->vstash.amax;
      if (xpol >= 0) {
        c->vstash.pol = xpol;
        c->vstash.args = *a;
        c->vstash.args.pol = xpol;
        c->vstash.tot = tot;
        c->vstash.amax = amM2;
        c->vstash.counts = counts;
        c->vstash.maxp = maxp;
        c->vstash.n_inter = n_inter;
        c->vstash.wmax = wmax;
        c->vstash.winsum = winsum;
        stashed = true;
      }
      if (!two) amM2 = amM;
      RPA_TRY(accumulate_tc(c, P, n_inter, wmax, Mf, Mf2, amM, amM2, cmax));
      if (cplx) RPA_TRY(qeff_f32(c, n_inter, (int)tot, Mf, Mf2));
    } else {
      cudaEventRecord(c->ev[2], c->stream);
      RPA_TRY(vertices_fp64(c, P, k0, nk, maxp, tot));
      cudaEventRecord(c->ev[3], c->stream);
      RPA_TRY(accumulate_fp64(c, P, n_inter, wmax));
      if (cplx) RPA_TRY(qeff_fp64(c, P, n_inter, (int)tot));
    }
    cudaEventRecord(c->ev[4], c->stream);
    RPA_CUDA(c, cudaStreamSynchronize(c->stream));
    t_pairs += elapsed(c, 1, 2);
    t_vert += elapsed(c, 2, 3);
    t_acc += elapsed(c, 3, 4);
    st_trans += (double)n_inter;
    st_win += winsum;
    st_launch += 1;
    for (int i = 0; i < nk; ++i) {
      int K1 = c->h_kmap[5 * (size_t)(k0 + i)];
      st_mac += (double)counts[k0 + i] * c->nlf * (c->legacy ? P.nsum_legacy : c->h_npw[K1]);
    }
    k0 = k1;
  }
  if (c->precision == RPA_PREC_MIXED && !c->defer_acc) RPA_TRY(df_to_f64(c, s_bytes / sizeof(double), P.nw, cplx));
  cudaEventRecord(c->ev[5], c->stream);
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  {
    int fl[4] = {0, 0, 0, 0};
    RPA_CUDA(c, cudaMemcpy(fl, c->d_flags.p, sizeof(int) * 4, cudaMemcpyDeviceToHost));
    if (fl[2]) return fail(c, RPA_ETIMEOUT, "rpa_chi0: a tensor-core completion wait timed out");
  }
  c->vstash.valid = stashed;
  c->stage_ms[0] = t_pairs;
  c->stage_ms[1] = t_vert;
  c->stage_ms[2] = t_acc;
  c->stats[0] = st_trans;
  c->stats[1] = st_win;
  c->stats[2] = st_mac;
  c->stats[3] = st_launch;
  c->last_mode = a->mode;
  c->last_no = a->no;
  c->last_nw = P.nw;
  c->last_domega = a->domega;
  c->last_Gcar = a->Gcar;
  c->have_S = true;
  c->have_chi0 = false;
  c->have_W = false;
  // results to the host, in the Fortran layouts
  double t_io = 0;
  if (S0_out || Qeff_out) {
    cudaEventRecord(c->ev[6], c->stream);
    if (S0_out) {
      RPA_TRY(ensure(c, c->d_tmp, s_bytes));
      launch_transpose_wp_to_fortran(c->d_S.as<double>(), c->d_tmp.as<double>(), P.nw, np, cplx ? 2 : 1, c->stream);
      RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
      RPA_TRY(copy_d2h(c, S0_out, c->d_tmp.p, s_bytes));
    }
    if (Qeff_out && cplx)
      RPA_CUDA(c, cudaMemcpyAsync(Qeff_out, c->d_Q.p, sizeof(double2) * np, cudaMemcpyDeviceToHost, c->stream));
    cudaEventRecord(c->ev[7], c->stream);
    RPA_CUDA(c, cudaStreamSynchronize(c->stream));
    t_io = elapsed(c, 6, 7);
  }
  c->stage_ms[5] = t_io;
  return RPA_OK;
}

int rpa_kk(rpa_ctx* c, int variant, double* chi0_out) {
  if (!c) return fail(c, RPA_EINVAL, "rpa_kk: ctx is NULL");
  if (!c->have_S) return fail(c, RPA_ESTATE, "rpa_kk: no S0 on the device (call rpa_chi0 first)");
  if (variant != RPA_KK_OPTABS_COMPLEX && variant != RPA_KK_SLOSS_REAL)
    return fail(c, RPA_EINVAL, "rpa_kk: unknown variant %d", variant);
  if ((variant == RPA_KK_OPTABS_COMPLEX) != (c->last_mode == RPA_MODE_CURRENT))
    return fail(c, RPA_EINVAL, "rpa_kk: variant does not match the S0 on the device");
  cudaSetDevice(c->device);
  cudaEventRecord(c->ev[0], c->stream);
  RPA_TRY(kk_run(c, variant, c->last_no, c->last_domega));
  cudaEventRecord(c->ev[1], c->stream);
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  c->stage_ms[3] = elapsed(c, 0, 1);
  c->have_chi0 = true;
  c->have_W = false;
  if (chi0_out) {
    const int nwo = c->last_no - 1, np = c->nlf * c->nlf;
    RPA_TRY(ensure(c, c->d_tmp, sizeof(double2) * (size_t)nwo * np));
    cudaEventRecord(c->ev[6], c->stream);
    launch_transpose_wp_to_fortran(c->d_chi0.as<double>(), c->d_tmp.as<double>(), nwo, np, 2, c->stream);
    RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
    RPA_TRY(copy_d2h(c, chi0_out, c->d_tmp.p, sizeof(double2) * (size_t)nwo * np));
    cudaEventRecord(c->ev[7], c->stream);
    RPA_CUDA(c, cudaStreamSynchronize(c->stream));
    c->stage_ms[5] = elapsed(c, 6, 7);
  }
  return RPA_OK;
}

int rpa_dyson(rpa_ctx* c, double c0, double eps, double* WT_out, double* epsinv_out, double* head_out) {
  if (!c) return fail(c, RPA_EINVAL, "rpa_dyson: ctx is NULL");
  if (!c->have_chi0) return fail(c, RPA_ESTATE, "rpa_dyson: no chi0 on the device (call rpa_kk first)");
  if (!(c0 > 0)) return fail(c, RPA_EINVAL, "rpa_dyson: c0 must be > 0");
  cudaSetDevice(c->device);
  std::vector<double> V;
  genV_host(c, c->last_Gcar, c0, eps, V);
  int nsing = 0, nzero = 0;
  const double2* head = nullptr;
  cudaEventRecord(c->ev[0], c->stream);
  RPA_TRY(dyson_fp64(c, V.data(), epsinv_out != nullptr, &nsing, &nzero, &head));
  cudaEventRecord(c->ev[1], c->stream);
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  c->stage_ms[4] = elapsed(c, 0, 1);
  const int nwo = c->last_no - 1, np = c->nlf * c->nlf;
  cudaEventRecord(c->ev[6], c->stream);
  if (head_out)
    RPA_CUDA(c, cudaMemcpyAsync(head_out, head, sizeof(double2) * nwo, cudaMemcpyDeviceToHost, c->stream));
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  if (WT_out || epsinv_out) {
    // d_tmp is reused for the transposes; heads were copied above
    RPA_TRY(ensure(c, c->d_tmp, sizeof(double2) * (size_t)nwo * np));
    if (WT_out) {
      launch_transpose_wp_to_fortran(c->d_WT.as<double>(), c->d_tmp.as<double>(), nwo, np, 2, c->stream);
      RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
      RPA_TRY(copy_d2h(c, WT_out, c->d_tmp.p, sizeof(double2) * (size_t)nwo * np));
    }
    if (epsinv_out) {
      launch_transpose_wp_to_fortran(c->d_eps.as<double>(), c->d_tmp.as<double>(), nwo, np, 2, c->stream);
      RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
      RPA_TRY(copy_d2h(c, epsinv_out, c->d_tmp.p, sizeof(double2) * (size_t)nwo * np));
    }
  }
  cudaEventRecord(c->ev[7], c->stream);
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  c->stage_ms[5] = elapsed(c, 6, 7);
  if (nsing) return fail(c, RPA_ESINGULAR, "singular matrix in gjel at %d frequencies", nsing);
  c->have_W = true;
  if (nzero && c->verbose) fprintf(stderr, "rpa_dyson: singular matrix in gjel (zero pivot) at %d frequencies\n", nzero);
  return RPA_OK;
}

int rpa_gfast(rpa_ctx* c, int ik, int ngd, int* out) {
  if (!c || !out) return fail(c, RPA_EINVAL, "rpa_gfast: bad arguments");
  if (c->ntot == 0 || !c->have_q) return fail(c, RPA_ESTATE, "rpa_gfast: k map and q must be set first");
  if (ik < 1 || ik > c->ntot) return fail(c, RPA_EINVAL, "rpa_gfast: ik outside 1..Ntot");
  if (c->legacy && ngd < 1) return fail(c, RPA_EINVAL, "rpa_gfast: NGd must be >= 1 without an igk map");
  cudaSetDevice(c->device);
  return build_gfast(c, ik - 1, ngd, out);
}

int rpa_init_igk(int nks, const double* xk, int npwx, int ngm, const double* g, double gcutw, int* igk_k, int* ngk) {
  if (nks <= 0 || !xk || npwx <= 0 || ngm <= 0 || !g || !igk_k || !ngk) return RPA_EINVAL;
  std::vector<double> gk(npwx);
  for (int ik = 0; ik < nks; ++ik) {
    int rc = gk_sort_host(xk + 3 * (size_t)ik, npwx, ngm, g, gcutw, &ngk[ik], igk_k + (size_t)npwx * ik, gk.data());
    if (rc != 0) return RPA_EINVAL;
  }
  return RPA_OK;
}

int rpa_kk_matrix(int variant, int no, double domega, double* K) {
  if (!K || no < 3 || !(domega > 0)) return RPA_EINVAL;
  if (variant != RPA_KK_OPTABS_COMPLEX && variant != RPA_KK_SLOSS_REAL) return RPA_EINVAL;
  std::vector<double> k;
  int nw = 0;
  kk_matrix(variant, no, domega, k, &nw);
  std::memcpy(K, k.data(), sizeof(double) * k.size());
  return RPA_OK;
}

int rpa_stage_times(const rpa_ctx* c, double* ms6) {
  if (!c || !ms6) return RPA_EINVAL;
  for (int i = 0; i < 6; ++i) ms6[i] = c->stage_ms[i];
  return RPA_OK;
}

int rpa_accum_tile(const rpa_ctx* c, int* gb, int* nio) {
  if (!c || !gb || !nio) return RPA_EINVAL;
  *gb = c->acc_last_gb;
  *nio = c->acc_last_nio;
  return RPA_OK;
}

int rpa_chi0_stats(const rpa_ctx* c, double* out4) {
  if (!c || !out4) return RPA_EINVAL;
  for (int i = 0; i < 4; ++i) out4[i] = c->stats[i];
  return RPA_OK;
}

int rpa_selftest(int which, double* result) {
  if (!result || which < 0 || which > 4) return RPA_EINVAL;
  if (which == 3) return selftest_wait(result);
  if (which == 4) return selftest_umma_ts(result);
  return selftest_umma(which, result);
}

int rpa_launch_count(const rpa_ctx* c, long long* count) {
  if (!c || !count) return RPA_EINVAL;
  *count = c->launches;
  return RPA_OK;
}

int rpa_get_stream(const rpa_ctx* c, void** stream) {
  if (!c || !stream) return RPA_EINVAL;
  *stream = (void*)c->stream;
  return RPA_OK;
}

int rpa_basis_info(const rpa_ctx* c, int* out4) {
  if (!c || !out4) return RPA_EINVAL;
  out4[0] = c->nks;
  out4[1] = c->nbnd;
  out4[2] = c->npwx;
  out4[3] = c->ng;
  return RPA_OK;
}

int rpa_synchronize(rpa_ctx* c) {
  if (!c) return RPA_EINVAL;
  cudaSetDevice(c->device);
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  return RPA_OK;
}

}  // extern "C"
