// rpa_internal.cuh -- shared state and helpers of the GB300 RPA library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <map>
#include <vector>

#include "../../include/rpa_gpu.h"

namespace rpa {

// ---------------------------------------------------------------------------
// Device buffer that only grows.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  template <class T>
  T* as() const { return reinterpret_cast<T*>(p); }
};

// One transition (n, m) of one FBZ k-point that contributes to S0 or Qeff.
// e1 = E(K1,n), e2 = E(K2,m) are kept apart so that dE = (o + e1) - e2 is
// formed in the reference's operation order (Sloss.f90:410, Optabs.f90:391).
struct Trans {
  int k;      // FBZ index within the current k-chunk
  int nm;     // n | (m << 16), 0-based bands
  int lo;     // first frequency row of the Lorentzian window (row index)
  int hi;     // last frequency row (inclusive)
  double e1;
  double e2;
  double c;   // prefactor: S0 += c * L(io) * M conj(M2) (inter) or Qeff += c M conj(M2) (intra)
};

static constexpr int KEY_INTRA = 0x7fffffff;

}  // namespace rpa

namespace rpa {
struct CopyPool;
}

// page-locked staging ring, copy threads and copy stream of a context's large
// host transfers (created on first use)
struct RpaHostIo {
  void* ring[2] = {nullptr, nullptr};
  cudaEvent_t ev[4] = {};
  cudaStream_t copy_stream = nullptr;
  rpa::CopyPool* pool = nullptr;
};

struct rpa_ctx {
  int device = 0;
  int precision = RPA_PREC_FP64;
  int verbose = 0;
  bool split_f16 = true;  // mixed path: fp16 (scaled) or bf16 hi/lo operands
  int tc_seg = 1;         // mixed path: chunks per TMEM accumulation segment
  int vertex_kind = 0;    // mixed-path vertices: 0 tensor cores (MN-major), 1 FP32 CUDA cores (chosen by the caller)
  cudaStream_t stream = nullptr;
  std::string err;
  // a context made by rpa_create_shared borrows the G list, symmetry and basis
  // buffers of its parent (read-only); the parent counts its live children
  rpa_ctx* parent = nullptr;
  int children = 0;

  // G list
  int ng = 0;
  std::vector<int> h_miller;  // 3*ng
  std::vector<double> h_G;    // 3*ng
  double KC[9] = {0};
  int box_lo[3] = {0, 0, 0}, box_dim[3] = {0, 0, 0};
  rpa::DevBuf d_miller, d_G, d_box;

  // symmetry (crystal-coordinate integer matrices, row-major [isym][3][3])
  int nsym = 0;
  std::vector<double> h_R, h_RI;  // Fortran R(48,3,3)
  std::vector<int> h_Rc, h_RIc;   // 48*9
  rpa::DevBuf d_Rc, d_RIc, d_Rcart;

  // basis
  int nks = 0, nbnd = 0, npwx = 0;
  bool legacy = false;
  std::vector<int> h_npw;
  std::vector<double> h_E;        // [k][b]
  int nbp = 0;                    // bands rounded up to 8 (coefficient planes)
  rpa::DevBuf d_npw, d_gidx, d_inv, d_coeff, d_coeff32, d_cpl, d_E;

  // k map
  int ntot = 0;
  std::vector<int> h_kmap;        // 5*ntot: K1,R1,K2,R2,iG0 (0-based)
  std::vector<double> h_ktot;
  rpa::DevBuf d_kmap, d_ktot;

  // q
  bool have_q = false;
  double q[3] = {0, 0, 0};
  int nlf = 0;
  std::vector<int> h_ilf, h_parG;
  rpa::DevBuf d_lf_miller, d_Glf;

  // per-call scratch
  rpa::DevBuf d_occ, d_counts, d_offsets, d_trans, d_keys, d_keys_alt, d_vals, d_vals_alt, d_sorted,
      d_M, d_M2, d_Mf, d_Mf2, d_tiles, d_tilesA, d_gmap, d_ginv, d_vbt, d_ybt, d_ptab, d_order, d_cub, d_wmax, d_ntrans,
      d_pairscr;
  // cached Gfast map (int16) of the last k-chunk, valid until the basis, k map or q change
  bool gmap_valid = false;
  int gmap_k0 = 0, gmap_nk = 0, gmap_nsum = 0, gmap_legacy_n = 0;
  // cached inverse map (gathered K1 plane wave of each K2 plane wave), same validity
  bool ginv_valid = false;
  int ginv_k0 = 0, ginv_nk = 0, ginv_nsum = 0;
  // rpa_chi0_prefetch: the polarisation whose vertices the next current-mode
  // chi0 computes beside its own (-1 none), and those vertex rows, kept in d_Mf2
  // for the chi0 call that directly follows with the same arguments
  int prefetch_pol = -1;
  struct VStash {
    bool valid = false;
    int pol = -1;
    rpa_chi0_args args{};
    long long tot = 0;
    float amax = 0.f;
    std::vector<int> counts;  // transitions per FBZ k-point
    int maxp = 0, n_inter = 0, wmax = 0;
    double winsum = 0.0;
  } vstash;
  // results
  int last_mode = -1, last_no = 0, last_nw = 0;
  double last_domega = 0.0, last_Gcar = 0.0;
  bool have_S = false, have_chi0 = false, have_W = false;
  // mixed-path vertex configuration: band-window width of the sequential side
  // (0: default) and gathered side for charge vertices (-1: fewer bands, 0:
  // empty bands through Gfast, 1: occupied bands through the inverse map); the
  // choice of the running rpa_chi0 call and the table that rpa_autotune fills,
  // keyed by (mode, nbnd, nocc, NGloc / 32)
  struct VtxTune {
    int ymax = 0, swap = -1;
    double ms = 0.0;
  };
  VtxTune vt_cur;
  bool vt_forced = false;
  std::map<long long, VtxTune> vt_table;
  // mixed-path accumulation tile (G-tile rows gb, frequency rows per CTA nio):
  // forced for every call (opts.reserved[2], or the autotuner's trial; gb = 0:
  // not forced) and the table rpa_autotune fills, keyed by (S0 kind, NGloc,
  // nw / 64); the variant the last accumulation used
  struct AccTune {
    int gb = 0, nio = 0;
    double ms = 0.0;
  };
  AccTune acc_force;
  std::map<long long, AccTune> acc_table;
  int acc_last_gb = 0, acc_last_nio = 0;
  // fixed KK kernels on the device, one slot per variant (Optabs, Sloss): FP64
  // and FP32 copies and the (no, domega) each was built for (no = 0: empty)
  int kk_key_no[2] = {0, 0};
  double kk_key_domega[2] = {0.0, 0.0};
  rpa::DevBuf d_kk[2], d_kkf[2];
  rpa::DevBuf d_S, d_Sdf, d_Q, d_chi0, d_kkw, d_V, d_eps, d_WT, d_flags, d_tmp;
  // the mixed-path accumulation of the running rpa_chi0 computed only the tile
  // pairs gi <= gj of S0 (M2 = M); the conversion to FP64 mirrors the rest
  bool s_sym = false;
  // deferred S0 accumulation (batch mode, batch.cu): with defer_acc set,
  // rpa_chi0 stops after the B-tile pre-split and leaves the accumulation's
  // launch description (an AccGroupItem) here for a grouped launch
  bool defer_acc = false;
  bool deferred = false;
  alignas(16) unsigned char deferred_item[256];
  int deferred_gb = 0, deferred_nio = 0, deferred_nw = 0;
  bool deferred_sepa = false, deferred_cplx = false;
  int s_gb = 96;  // G-tile rows of that accumulation
  double stage_ms[6] = {0, 0, 0, 0, 0, 0};
  long long launches = 0;  // kernels launched by this context
  double stats[4] = {0, 0, 0, 0};
  cudaEvent_t ev[8] = {};
  RpaHostIo io;
};

namespace rpa {

int fail(rpa_ctx* c, int code, const char* fmt, ...);
int cuda_fail(rpa_ctx* c, cudaError_t e, const char* what);
int ensure(rpa_ctx* c, DevBuf& b, size_t bytes);
void release(DevBuf& b);

#define RPA_CUDA(ctx, call)                                   \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return rpa::cuda_fail(ctx, e_, #call); \
  } while (0)

// Raises a kernel's dynamic shared-memory limit to the most the device allows
// next to the kernel's static shared memory.  Every caller sets the same value,
// so contexts that launch the kernel from several host threads (with sizes
// that depend on their own request) never lower the limit under another's
// launch.
template <class K>
inline cudaError_t allow_dynamic_smem(K kern, int device) {
  int optin = 0;
  cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  if (e != cudaSuccess) return e;
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, kern);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
}

#define RPA_TRY(...)                 \
  do {                               \
    int rc_ = (__VA_ARGS__);         \
    if (rc_ != RPA_OK) return rc_;   \
  } while (0)

// ---------------------------------------------------------------------------
// Stage entry points (implemented in the k_*.cu files).
struct Chi0Plan {
  int mode, pol, no, nw, wbase;  // nw = rows of S0 (no or 2no+1); row r <-> io = r + wbase
  int nocc, nsum_legacy;
  double domega, eta, cut, df_cut, T, Efermi, norm_s, norm_q, Gcar;
  int ntot_norm;
};

int build_gfast(rpa_ctx* c, int ik, int nsum_legacy, int* out);

// tile variants (G-tile rows, frequency rows per CTA) of the warp-specialised
// accumulation for the complex or real S0; returns their number
int acc_variant_list(bool cplx, int* gb, int* nio, int cap);

// key of the accumulation tuning table: (S0 kind, NGloc, nw / 64)
inline long long acc_tune_key(bool cplx, int nlf, int nw) {
  return (long long)(cplx ? 1 : 0) | ((long long)nlf << 1) | ((long long)(nw / 64) << 16);
}

// key of the vertex tuning table: (mode, nbnd, nocc, NGloc / 32)
inline long long vtx_tune_key(int mode, int nbnd, int nocc, int nlf) {
  return (long long)mode | ((long long)nbnd << 4) | ((long long)nocc << 20) | ((long long)(nlf / 32) << 36);
}
int kk_apply_real_fp64(rpa_ctx* c, DevBuf& buf, const std::vector<double>& K, int nrow, int nw, const double* S,
                       double2* out, int np, bool pi_epilogue);

// large host transfers (host_io.cu): synchronous device -> host copy through
// the page-locked ring when dst is pageable; basis upload overlapping copies
// and transposes; release of the ring, threads and copy stream
int copy_d2h(rpa_ctx* c, void* dst, const void* src, size_t bytes);
// V (genV) of the context's q-point and local fields, real (nlf, nlf) column-major
void genV_of(const rpa_ctx* c, double c0, double eps, std::vector<double>& V);
int upload_basis(rpa_ctx* c, const double* coeff, int nks, int nbnd, int npwx, double2* dst);
int host_io_prepare(rpa_ctx* c);
void host_io_release(rpa_ctx* c);
void launch_basis_transpose(const double2* src, double2* dst, int nkc, int nbnd, int npwx, cudaStream_t s);

// device layout transposes between [w][p] (library) and (w fastest) Fortran
void launch_transpose_wp_to_fortran(const double* src, double* dst, int nw, int np, int ncomp,
                                    cudaStream_t s);

}  // namespace rpa
