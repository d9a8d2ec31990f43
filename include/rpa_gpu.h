/* rpa_gpu.h -- C ABI of the GB300 RPA response library.
 *
 * Drop-in for the OpenMP k-loop, the Kramers-Kronig stage and the Dyson
 * stage of the 2DMaterialsOpticalProps drivers:
 *   Chi_RPA/Optabs.f90:291-471  (current vertices, complex S0 and Qeff)
 *   Chi_RPA/Optabs.f90:575-614  (KK of complex S0 -> chi0 / Pi)
 *   W/Sloss.f90:309-438         (charge vertices, real S0)
 *   W/Sloss.f90:452-481         (KK, V, eps = 1 - chi0 V, gjel, chi, W)
 * The drivers keep their namelists, the setup (PointR, genFBZ, findKinIBZ,
 * findKQinBZ, genGlf) and every file they write; they hand the arrays they
 * already hold to these calls through an ISO_C_BINDING interface.
 *
 * Conventions
 *  - Every array is Fortran column-major, exactly as the drivers declare it;
 *    every index handed in (K1, R1, K2, R2, iG0, igk, ilf) is 1-based.
 *  - Complex arrays are interleaved (re, im) doubles (Fortran complex(dp)).
 *  - Host buffers are owned by the caller and only touched during the call.
 *    Device state (coefficients, energies, index maps, S0, chi0, W) is owned
 *    by the context and released by rpa_destroy.
 *  - Every call returns RPA_OK (0) or a negative error code and never exits
 *    the process; rpa_last_error() gives the message.  One context per host
 *    thread; calls on a context are serialised by the caller.
 */
#ifndef RPA_GPU_H
#define RPA_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define RPA_OK 0
#define RPA_EINVAL (-1)     /* bad argument or size (e.g. NGd > igwx, Nlf > capacity) */
#define RPA_ENOMEM (-2)     /* device allocation failed */
#define RPA_ESINGULAR (-3)  /* gjel met a repeated pivot ("singular matrix in gjel" + stop) */
#define RPA_ETIMEOUT (-4)   /* a bounded device wait gave up */
#define RPA_ECUDA (-5)      /* CUDA runtime error */
#define RPA_ESTATE (-6)     /* call made before the state it needs was set */
#define RPA_ENOTFOUND (-7)  /* an index map could not be resolved */

enum { RPA_PREC_FP64 = 0, RPA_PREC_MIXED = 1 };
enum { RPA_MODE_CHARGE = 0, RPA_MODE_CURRENT = 1 };
enum { RPA_POL_XX = 0, RPA_POL_YY = 1, RPA_POL_ZZ = 2, RPA_POL_YZ = 3, RPA_POL_ZY = 4 };
enum { RPA_KK_OPTABS_COMPLEX = 1, RPA_KK_SLOSS_REAL = 2 };

typedef struct rpa_ctx rpa_ctx;

typedef struct rpa_opts {
  int device;     /* CUDA device ordinal */
  int precision;  /* RPA_PREC_FP64 (plain drop-in) or RPA_PREC_MIXED */
  int verbose;    /* 0: silent */
  int split;      /* RPA_PREC_MIXED operand split: 0 = fp16 hi/lo with power-of-two
                     scaling (default, ~2^-22 per operand), 1 = bf16 hi/lo (~2^-16) */
  int reserved[4]; /* reserved[0]: mixed path, chunks of 32 transitions summed in one
                      TMEM accumulator before read-back (0 -> 1); keep 0.
                      reserved[1]: mixed-path vertex kernel, 0 = tensor cores with
                      MN-major operands (default; at most 32767 plane waves and
                      181 bands per k-point, else rpa_load_basis returns
                      RPA_EINVAL), 1 = FP32 CUDA cores (any basis size).
                      reserved[2]: mixed-path S0 accumulation tile for every
                      call with M2 = M, gb | nio << 8 (gb local fields per
                      G-tile, nio frequency rows per CTA; 0 = the autotuner's
                      table, else a cost model).  Variants: complex S0 (96, 1)
                      (64, 1) (32, 2); real S0 (96, 2) (128, 1) (64, 2) (48, 2)
                      (32, 2); another value makes rpa_chi0 return RPA_EINVAL. */
} rpa_opts;

/* Arguments of one chi0 accumulation (the namelist values the drivers use).
 * Energies are in Hartree, as the drivers hold them after their eV->Ha
 * conversion (Optabs.f90:173-181, Sloss.f90:195-199). */
typedef struct rpa_chi0_args {
  int mode;       /* RPA_MODE_CHARGE: Sloss (n <= nocc < m, real S0, io = 1..no)
                     RPA_MODE_CURRENT: Optabs (df cut, complex S0, io = -no..no, Qeff) */
  int pol;        /* RPA_POL_* (current vertices, genStrujniVrhovi) */
  int ngd;        /* NGd: coefficients summed per band when the basis has no igk
                     map (legacy drivers); ignored with an igk map (npw(K1) is used) */
  int nocc;       /* Sloss Nocc */
  int no;         /* number of frequencies */
  int ntot_norm;  /* Ntot in the 1/(pi Ntot Vcell) normalisation; 0 -> ntot of rpa_kmap */
  double domega;  /* Hartree */
  double eta;     /* Sloss eta / Optabs eta_inter, Hartree */
  double lor_cut; /* Optabs Lor_cut (Sloss hard-codes 1e-3) */
  double df_cut;  /* Optabs df_cut */
  double T;       /* Optabs temperature, Hartree */
  double Efermi;  /* Optabs Fermi energy, Hartree */
  double Vcell;   /* bohr^3 */
  double Gcar;    /* 2 pi / a0 */
} rpa_chi0_args;

/* Replaces: the process-wide setup of a driver run.  Creates a context on
 * opts->device with its own stream. */
int rpa_create(rpa_ctx** out, const rpa_opts* opts);

/* Releases every device buffer of the context. */
int rpa_destroy(rpa_ctx* ctx);

/* Message of the last failing call on ctx (or of rpa_create when ctx is NULL). */
const char* rpa_last_error(const rpa_ctx* ctx);

/* Replaces: loadKC + loadG (Optabs.f90:652-680, 1061-1110; Sloss.f90:1309-1348).
 *   miller : Gi(3,NG), the crystal (Miller) coordinates read from gvectors.xml
 *   G      : G(3,NG), Cartesian in 2pi/a0 units, as loadG computes it
 *   KC     : KC(3,3), reciprocal axes (columns b1, b2, b3) in 2pi/a0 units
 * G(:,1) must be 0 (loadG stops otherwise). */
int rpa_set_gvectors(rpa_ctx* ctx, int ng, const int* miller, const double* G, const double* KC);

/* Replaces: PointR (Chi_RPA/PointR.f90:11-144) output R(48,3,3), RI(48,3,3)
 * in Cartesian coordinates.  Each operation must map the G lattice onto
 * itself (integer matrix in crystal coordinates). */
int rpa_set_symmetry(rpa_ctx* ctx, int nsym, const double* R, const double* RI);

/* Replaces: the per-band coefficient reads inside the k-loop
 * (iotk_scan_dat, Optabs.f90:332-374, Sloss.f90:355-393) and loadkIandE.
 *   npw   : npw(nks) = igwx of each IBZ k-point
 *   igk   : igk_k(npwx,nks) (1-based into G, init_igk of Modules/qe_gksort.f90),
 *           or NULL for the legacy drivers, where coefficient i belongs to G(:,i)
 *   coeff : C(npwx,nbnd,nks) complex(dp)
 *   E     : E(nks,nbnd) Hartree (any scissor already applied)
 * The basis stays resident on the device until the next call or rpa_destroy.
 * coeff may be ordinary (pageable) memory — it then passes through the
 * context's page-locked staging ring — or page-locked / device memory, which
 * is copied directly; the same holds for the large outputs of rpa_chi0,
 * rpa_kk and rpa_dyson. */
int rpa_load_basis(rpa_ctx* ctx, int nks, int nbnd, int npwx, const int* npw, const int* igk,
                   const double* coeff, const double* E);

/* Replaces: findKinIBZ / findKQinBZ results of the k-loop
 * (Optabs.f90:306,320; Sloss.f90:327,339): for every FBZ point ik,
 * ktot(3,ik) = R1*K1 and ktot + q = G(iG0) + R2*K2. */
int rpa_kmap(rpa_ctx* ctx, int ntot, const double* ktot, const int* K1, const int* R1,
             const int* K2, const int* R2, const int* iG0);

/* ---- k-point bookkeeping on the device --------------------------------------
 * The drivers' O(Ntot^2) / O(NG Ntot Nsym NkI) host searches, with identical
 * results (first-match order and eps tests of the reference loops).  They use
 * the symmetry of rpa_set_symmetry (identity when never called) and, for
 * rpa_find_kq, the G list of rpa_set_gvectors.  k-points are Cartesian, 2pi/a0
 * units; kI(3,nki), ktot(3,ntot) column-major; index outputs are 1-based, as
 * rpa_kmap takes them.
 *
 * Replaces: genFBZ (Chi_RPA/Optabs.f90:886-933; Sloss keeps its own copy).
 * Writes the *ntot distinct points R_i kI_j (i outer) into ktot; RPA_EINVAL when
 * more than max_ntot. */
int rpa_gen_fbz(rpa_ctx* ctx, int nki, const double* kI, double eps, int max_ntot, int* ntot, double* ktot);

/* Replaces: findKinIBZ (Chi_RPA/Optabs.f90:776-818) for every FBZ point.
 * RPA_ENOTFOUND ("Can not find wave vector K= in I.B.Z.") when a point has no
 * image. */
int rpa_find_k_ibz(rpa_ctx* ctx, int ntot, const double* ktot, int nki, const double* kI, double eps, int* R1,
                   int* K1);

/* Replaces: findKQinBZ (Chi_RPA/Optabs.f90:820-884) for every FBZ point k and
 * k + q.  RPA_ENOTFOUND when a K+Q has no (G, FBZ point, IBZ image) match. */
int rpa_find_kq(rpa_ctx* ctx, int ntot, const double* ktot, int nki, const double* kI, const double* q, double eps,
                int* iG0, int* R2, int* K2);

/* ---- Tile autotuner (mixed path; no counterpart in the reference) -----------
 * Runs the chi0 call of args on the current k map and q once per candidate
 * tensor-core vertex configuration (band-window width of the sequential side;
 * for charge vertices also the gathered side) and keeps the fastest for later
 * rpa_chi0 calls with the same (mode, nbnd, nocc, NGloc / 32); *best_ms (may be
 * NULL) = its vertex-stage time.  Then, with that vertex configuration, it runs
 * every S0 accumulation tile variant (see opts.reserved[2]; S0 with M2 = M)
 * and keeps the fastest accumulation stage for calls with the same (S0 kind,
 * NGloc, nw / 64).  Shared contexts start with their parent's tables.
 * RPA_ESTATE on an FP64 context or with reserved[1] != 0. */
int rpa_autotune(rpa_ctx* ctx, const rpa_chi0_args* args, double* best_ms);

/* The tables as JSON text ({"vertex": [{"mode", "nbnd", "nocc", "nlf32", "ymax",
 * "swap", "ms"}, ...], "accum": [{"cplx", "nlf", "nw64", "gb", "nio", "ms"},
 * ...]}); *len = bytes needed including the NUL (buf may be NULL to query it). */
int rpa_tune_export(const rpa_ctx* ctx, char* buf, int cap, int* len);

/* Replaces the tables by the ones in json (as written by rpa_tune_export; the
 * "accum" list may be absent). */
int rpa_tune_import(rpa_ctx* ctx, const char* json);

/* ---- On-disk formats (host only, no context; errors via rpa_last_error(NULL)) --
 *
 * Replaces: loadG (Modules/io_qe.f90:11-71).  Reads the Miller indices of
 * <savedir>/charge-density.dat (QE 6 binary), G(:,iG) = KC mill(:,iG)
 * (KC(3,3) column-major, 2pi/a0 units) and parG(iG) = mill(3,iG) (parG may be
 * NULL).  miller(3,max_ng), G(3,max_ng) column-major. */
int rpa_qe_read_gvectors(const char* savedir, const double* KC, int max_ng, int* ng, int* miller, double* G,
                         int* parG);

/* Header of <savedir>/wfc<ik>.dat: igwx, npol, nbnd and xk(3) (xk may be NULL). */
int rpa_qe_wfc_info(const char* savedir, int ik, int* igwx, int* npol, int* nbnd, double* xk);

/* Replaces: loadCs_full (Modules/io_qe.f90:124-166).  The first nbnd bands of
 * <savedir>/wfc<ik>.dat into coeff(npwx, nbnd) complex(dp) column-major (zero
 * beyond igwx), and the record of Miller indices into miller(3, igwx) (may be
 * NULL).  npol must be 1. */
int rpa_qe_read_wfc(const char* savedir, int ik, int npwx, int nbnd, double* coeff, int* miller);

/* Replaces: the calc = 1 output of Optabs (Chi_RPA/Optabs.f90:482-508):
 * S0(-no:no,nlf,nlf) and Qeff(nlf,nlf) complex(dp) column-major as text, one
 * 'omega=' line per frequency and '(2F15.10)' per element (path_qeff / Qeff may
 * be NULL). */
int rpa_write_corrfun(const char* path_s0, const char* path_qeff, int no, int nlf, double domega, const double* S0,
                      const double* Qeff);

/* Replaces: the calc = 2 read-back (Chi_RPA/Optabs.f90:531-559) of those files. */
int rpa_read_corrfun(const char* path_s0, const char* path_qeff, int no, int nlf, double* S0, double* Qeff);

/* Replaces: writeWT_Qi (W/Sloss.f90:1572-1601).  The first frequency of
 * WT(no_rows,nlf,nlf) complex(dp) column-major, '(10F15.5)'. */
int rpa_write_wt(const char* path, int no_rows, int nlf, double domega, const double* WT);

/* Replaces: findMinQ + genGlf/genGlfandParity results (Optabs.f90:272,248;
 * Sloss.f90:295,258).
 *   q    : q(3), 2pi/a0 units (before the Gcar conversion)
 *   ilf  : ilf(nlf), 1-based G index of each local field (Glf(:,i) = G(:,ilf(i)))
 *   parG : parG(nlf) = +-1 parity used by genV (may be NULL for Optabs) */
int rpa_set_q(rpa_ctx* ctx, const double* q, int nlf, const int* ilf, const int* parG);

/* Replaces: the OpenMP k-loop with its vertices and the S0 accumulation,
 * Optabs.f90:291-471 (mode CURRENT) or Sloss.f90:309-438 (mode CHARGE).
 * S0_out: CURRENT -> complex S0(-no:no,nlf,nlf); CHARGE -> real S0(no,nlf,nlf).
 * Qeff_out: complex Qeff(nlf,nlf) (CURRENT only).  Either may be NULL, in which
 * case the result only stays on the device for rpa_kk. */
int rpa_chi0(rpa_ctx* ctx, const rpa_chi0_args* args, double* S0_out, double* Qeff_out);

/* No counterpart in the reference (each Optabs run computes one polarisation,
 * Optabs.f90:291-471).  RPA_PREC_MIXED, current mode: the next rpa_chi0 on ctx
 * for a single-component polarisation (xx, yy, zz) also computes the vertices
 * of pol (another of RPA_POL_XX, YY, ZZ) in the same vertex pass -- the two
 * share the gathered coefficients and the c . c block -- and keeps them on the
 * device.  An rpa_chi0 for pol that directly follows that call on ctx with the
 * same arguments (rpa_kk and rpa_dyson in between are fine; rpa_set_q,
 * rpa_kmap, rpa_load_basis, rpa_set_gvectors, rpa_set_symmetry or another
 * rpa_chi0 drop them) uses them instead of computing its vertices.  Without
 * effect on the FP64 path, charge mode, the yz / zy pair, the CUDA-core vertex
 * kernel and transitions that need more than one k chunk.  One-shot: applies
 * to the next rpa_chi0 only; pol = -1 cancels.  Results equal those of the
 * two calls without it up to FP32 rounding order. */
int rpa_chi0_prefetch(rpa_ctx* ctx, int pol);

/* Replaces: genReChi0/genImChi0 (Optabs.f90:1112-1318, variant
 * RPA_KK_OPTABS_COMPLEX) or genChi0 (Sloss.f90:954-1059, RPA_KK_SLOSS_REAL)
 * for io = 1..no-1 over the S0 left on the device by rpa_chi0.
 * chi0_out: complex chi0(no-1,nlf,nlf) (may be NULL). */
int rpa_kk(rpa_ctx* ctx, int variant, double* chi0_out);

/* Replaces: the Dyson loop of Sloss.f90:452-481 for io = 1..no-1:
 * genV, eps = I - chi0 V, gjel (W/gjel.f), chi = eps^-1 chi0, WT = V + V chi V.
 * RPA_PREC_FP64 follows these steps; RPA_PREC_MIXED inverts eps in FP64 as
 * well but forms WT as V eps^-1, the same matrix (eps^-1 chi0 V = eps^-1 - I)
 * with one product and no cancellation between V and V chi V.
 *   c0, eps    : the &parameters c0 (bohr) and eps of the driver
 *   WT_out     : complex WT(no-1,nlf,nlf) (may be NULL)
 *   epsinv_out : complex eps^-1(no-1,nlf,nlf) (may be NULL)
 *   head_out   : complex eps^-1_{11}(no-1), the loss function is -Im (may be NULL)
 * Returns RPA_ESINGULAR where gjel would stop. */
int rpa_dyson(rpa_ctx* ctx, double c0, double eps, double* WT_out, double* epsinv_out,
              double* head_out);

/* Replaces: init_igk (Modules/qe_gksort.f90:11-42): igk_k(npwx,nks) and ngk(nks)
 * of the k+G spheres |k+G|^2 <= gcutw, sorted as hpsort_eps does.
 * Host-side; needs no device.  Returns RPA_EINVAL when npwx is too small or
 * the G list ends inside a sphere. */
int rpa_init_igk(int nks, const double* xk, int npwx, int ngm, const double* g, double gcutw,
                 int* igk_k, int* ngk);

/* Diagnostic for the index-map parity checks: the Gfast map of FBZ point ik
 * (1-based) in the reference's convention (Sloss.f90:905-944): for local
 * field iG and coefficient iG1 of K1, the 1-based K2 basis position of
 * G'' = RI_R2 (R_R1 G1 + Glf + G_iG0), or NG2+1 when K2 has no such
 * coefficient.  out is Gfast((iG-1)*nsum + iG1), nsum = NGd (no igk map) or
 * npw(K1). */
int rpa_gfast(rpa_ctx* ctx, int ik, int ngd, int* out);

/* Host-side diagnostic: the KK kernel matrix K((no-1), nw) that rpa_kk applies
 * (row-major, rows io = 1..no-1; columns are the S0 rows: jo = 1..no for
 * RPA_KK_SLOSS_REAL, j = -no..no for RPA_KK_OPTABS_COMPLEX).  Needs no device. */
int rpa_kk_matrix(int variant, int no, double domega, double* K);

/* Allocation-free Dyson step.  No counterpart in the reference: it serves
 * callers that cannot allocate device memory when they need the solve -- code
 * inside a host framework that owns every device allocation through its own
 * pool, or latency-critical serving code that cannot afford cudaMalloc/cudaFree
 * (which synchronise the device) per request.  It runs the same FP64 kernel as
 * rpa_dyson (eps = I - chi0 V, gjel, chi = eps^-1 chi0, WT = V + V chi V) on
 * device buffers the caller owns, with its workspace in a fixed 13.5 MiB device
 * array compiled into the library (held by every GPU that loads it, until the
 * process exits); it calls no allocating routine.
 *   chi0 : device, complex chi0 for nwo frequencies, [nwo][n*n], each n x n
 *          matrix column-major (the layout rpa_kk leaves on the device)
 *   V    : device, real V(n,n) column-major
 *   WT   : device, complex [nwo][n*n] output;  head: device, complex [nwo]
 *          output eps^-1_{11} (may be NULL)
 *   stream : cudaStream_t (as void*) the kernels are launched on
 *   n_singular : host; if not NULL the call waits for the stream and returns
 *          the number of frequencies where gjel would stop (RPA_ESINGULAR)
 * Limits: n <= 96 (RPA_EINVAL otherwise), any nwo >= 1.  The kernel runs on
 * at most 32 blocks (32 of the GPU's SMs, one frequency per block at a time),
 * which is what the fixed workspace holds.
 * Set-up: with CUDA's lazy module loading, the library's kernels and this
 * workspace are put on a device at the first launch from the library there
 * (any entry point) or at this call's first use on the device, which also
 * looks up the workspace's device address with that device current.  That
 * first call reserves the 13.5 MiB and can fail with RPA_ECUDA if the device
 * is full: make it at start-up, before a framework's memory pool takes the
 * device memory, and before any stream capture.  The address stays valid for
 * the device's primary context; after a cudaDeviceReset do not call this
 * entry point again in the same process.
 * Every call shares the one workspace: calls that overlap on the GPU race.
 * Uses the current device. */
int rpa_dyson_noalloc(const double* chi0, const double* V, int n, int nwo, double* WT, double* head,
                      void* stream, int* n_singular);

/* Replaces: the calc = 2 assembly of Optabs (Optabs.f90:575-614) on the chi0
 * and Qeff of the last Optabs rpa_chi0 + rpa_kk:
 *   Pi(io) = chi0(io) + Pi_dia + Qeff oi / (oi + i eta_intra),
 *   Pi_dia = -Re chi0(io = 1), oi = (io-1) domega, io = 1..no-1.
 *   pi11_out  : host, complex (no-1): Pi_tot(1,1), the spectrum the driver writes
 *   sigma_out : host, real (2, no-1): [inter, intra] conductivity in units of
 *               2 pi e^2 / h, Re(-i c0 Pi / oi), 0 at io = 1 (not written there);
 *               the interband term is Pi_tot(1,1) as the driver reads it after its
 *               (iG, jG) loop: with the intraband term when Nlf > 1, without it
 *               when Nlf = 1; the intraband term is Qeff(1,1) oi / (oi + i eta_intra)
 *   Pi_out    : host, complex Pi(no-1, Nlf, Nlf), or NULL
 * eta_intra in Hartree, c0 in bohr (namelist values). */
int rpa_pi(rpa_ctx* ctx, double eta_intra, double c0, double* pi11_out, double* sigma_out, double* Pi_out);

/* Replaces: the Kramers-Kronig transform of the screened interaction and its
 * self-check in Sloss (Sloss.f90:486-534 with genW1W2 :1062-1171 and
 * writeKramKron_Qi :1603-1641), on the W of the last rpa_dyson:
 *   S_W(io) = -Im WT(io) / pi for io < no, S_W(no) = S0(no) of the chi0 (the
 *   driver does not overwrite that row); W1, W2 as genW1W2;
 *   gamma_p_out : host, complex (no-1, Nlf, Nlf): Gamma+ = (W1, Im WT), or NULL
 *   gamma_m_out : host, complex (no-1, Nlf, Nlf): Gamma- = (-W2, 0), or NULL
 *   check5      : host, [0] KKS = int (WindKK - Wind)^2, [1] SKK = int Wind^2,
 *                 [2] 100 |KKS / SKK| (percent), [3] real Gamma+(o=0,1,1),
 *                 [4] real[WT(o=0,1,1) - V(1,1)] / 2, or NULL. */
int rpa_kk_w(rpa_ctx* ctx, double* gamma_p_out, double* gamma_m_out, double* check5);

/* Timing of the stages of the last rpa_chi0/rpa_kk/rpa_dyson calls (ms, CUDA
 * events on the context stream): [0] pairs+sort, [1] vertices,
 * [2] accumulation, [3] KK, [4] Dyson, [5] host<->device copies. */
int rpa_stage_times(const rpa_ctx* ctx, double* ms6);

/* Statistics of the last rpa_chi0: [0] transitions with a non-empty window,
 * [1] sum over transitions of window lengths (N_win), [2] vertex complex MACs,
 * [3] accumulation launches. */
int rpa_chi0_stats(const rpa_ctx* ctx, double* out4);

/* The S0 accumulation tile the last rpa_chi0 of a mixed context used: *gb
 * local fields per G-tile and *nio frequency rows per CTA (0, 0 on the FP64
 * path or when no interband transition contributed).  Diagnostic; no
 * counterpart in the reference. */
int rpa_accum_tile(const rpa_ctx* ctx, int* gb, int* nio);

/* On-device self-test of the tensor-core building blocks on the current
 * device: which = 0, 1, 2 runs a 128 x N x 192 bf16 tcgen05 GEMM (N = 192,
 * 96, 256) from swizzled shared-memory tiles into TMEM and stores in *result
 * its max relative deviation from an FP32 CUDA-core product of the same
 * values.  Returns RPA_ETIMEOUT if the bounded completion wait gave up.
 * which = 3 waits on an mbarrier that nothing arrives on: the bounded wait
 * gives up (a few milliseconds) and the call returns RPA_ETIMEOUT with *result
 * = the cycles waited, leaving the device usable.
 * which = 4 runs the 128 x 192 x 192 GEMM with f16 inputs and A in tensor
 * memory (tcgen05.mma with an [a_tmem] operand, two f16 of K per 32-bit
 * column, rows in lanes), B from a swizzled shared-memory tile. */
int rpa_selftest(int which, double* result);

/* Number of CUDA kernels this context has launched so far (its own kernels;
 * the radix sort's library kernels are not counted). */
int rpa_launch_count(const rpa_ctx* ctx, long long* count);

/* The cudaStream_t (as void*) every kernel of ctx is launched on, so that a
 * caller can order its own work or time the context with CUDA events. */
int rpa_get_stream(const rpa_ctx* ctx, void** stream);

/* Blocks until the context stream is idle. */
int rpa_synchronize(rpa_ctx* ctx);

/* Dimensions of the loaded basis: out4 = {nks, nbnd, npwx, ng} (zeros before
 * rpa_load_basis / rpa_set_gvectors). */
int rpa_basis_info(const rpa_ctx* ctx, int* out4);

/* ---- Several q-points on one resident basis --------------------------------
 * No counterpart in the reference: its drivers compute one q-point per process
 * and reread the wavefunctions each time. */

/* A context on parent's device that uses parent's G list, symmetry and basis
 * on the device without copying them, and has its own k map, q, per-call
 * buffers, results and stream.  Shared contexts driven from different host
 * threads run their kernels concurrently.  precision: RPA_PREC_FP64,
 * RPA_PREC_MIXED (needs a parent created with RPA_PREC_MIXED, which holds the
 * split coefficient copies) or -1 for the parent's.  parent must be a context
 * that loaded the basis itself; while shared contexts exist neither side may
 * call rpa_set_gvectors / rpa_set_symmetry / rpa_load_basis (RPA_ESTATE) and
 * rpa_destroy(parent) fails with RPA_ESTATE. */
int rpa_create_shared(rpa_ctx** out, rpa_ctx* parent, int precision);

/* Request loop with continuous batching.  A server owns nslots shared contexts
 * of parent and one worker thread each.  Submitted requests wait in a FIFO
 * queue; the head starts as soon as a worker is free and its device footprint
 * (about NGloc^2 x frequency rows complex values for S0, chi0 and, for W, the
 * Dyson buffers, plus the vertex rows) fits in mem_bytes next to the requests
 * already running; a request larger than mem_bytes runs alone.  Requests that
 * arrive while others run start without waiting for them to finish and their
 * kernels overlap on the GPU. */
typedef struct rpa_server rpa_server;
enum { RPA_REQ_CHI0 = 0, RPA_REQ_W = 1 };
typedef struct rpa_request {
  int kind;        /* RPA_REQ_CHI0: S0 (+ Qeff) and chi0 by KK; RPA_REQ_W: also the
                      Dyson solve, W and eps^-1_{11} (loss function) */
  int kk_variant;  /* RPA_KK_* */
  int ntot;        /* FBZ points and their maps, as rpa_kmap */
  const double* ktot;
  const int *K1, *R1, *K2, *R2, *iG0;
  double q[3];     /* as rpa_set_q */
  int nlf;
  const int* ilf;
  const int* parG;
  rpa_chi0_args args;
  double c0, eps;  /* as rpa_dyson (RPA_REQ_W) */
  double* S0_out;  /* host outputs as rpa_chi0 / rpa_kk / rpa_dyson; NULL = not wanted */
  double* Qeff_out;
  double* chi0_out;
  double* WT_out;
  double* head_out;
} rpa_request;
/* Every array a request points to must stay valid until rpa_server_wait
 * returns for it. */
int rpa_server_create(rpa_server** out, rpa_ctx* parent, int nslots, double mem_bytes);
int rpa_server_submit(rpa_server* srv, const rpa_request* req, long long* id);
/* Blocks until request id is done; returns its status.  times3 (may be NULL):
 * [0] latency from submission to completion, [1] time in the queue,
 * [2] service time, seconds. */
int rpa_server_wait(rpa_server* srv, long long id, double* times3);
/* Message of the last failed request returned by rpa_server_wait. */
const char* rpa_server_last_error(const rpa_server* srv);
/* Finishes the queued requests, stops the workers, destroys the contexts. */
int rpa_server_destroy(rpa_server* srv);

/* A server as rpa_server_create plus one batching worker (no counterpart in
 * the reference): when free, it takes up to batch_q queued W requests (charge
 * mode, Sloss KK, no S0 / Qeff / chi0 outputs) in arrival order, as many as fit
 * the budget next to the running requests, and runs them as one rpa_batch
 * (per-request setup, then one CUDA graph with the grouped-tile S0 launches and
 * every request's KK and Dyson).  The slot workers keep taking requests of
 * any kind.  parent must be RPA_PREC_MIXED (the batch's contexts are mixed). */
int rpa_server_create_batched(rpa_server** out, rpa_ctx* parent, int nslots, double mem_bytes, int batch_q);
/* Requests completed through the batching worker so far. */
int rpa_server_batched_count(const rpa_server* srv, long long* n);

/* ---- Batched W requests in one CUDA graph (no counterpart in the reference) --
 * A batch owns max_q shared contexts on parent's resident basis (parent must be
 * RPA_PREC_MIXED).  rpa_batch_run solves nq <= max_q W requests (RPA_REQ_W,
 * RPA_MODE_CHARGE, RPA_KK_SLOSS_REAL; outputs head_out and WT_out, host, or
 * NULL) as the Sloss q loop (Sloss.f90:292-481) would for each, in two parts:
 *   - per request, on its context: k map and q, pairs, windows, sort,
 *     tensor-core vertices, B-tile pre-split (the host decisions of a q-chain:
 *     transition counts, the window bound, operand scales), V, the KK matrix;
 *   - one CUDA graph, launched once: per S0 tile shape one grouped-tile launch
 *     of the S0 accumulation over every request of that shape (each request
 *     keeps its own NGloc, nw, transitions and buffers), then per request, as
 *     parallel branches, S0 to FP64, KK and the FP64 Dyson solve.
 * status[i] = the request's own result code; the call returns RPA_OK or the
 * first failing request's code (rpa_batch_last_error gives its message).  Each
 * request needs all its transitions in one k-chunk (RPA_EINVAL otherwise) and
 * the default split / segment options.  Arrays of reqs must stay valid during
 * the call.  The results equal rpa_chi0 + rpa_kk + rpa_dyson on a mixed
 * context to the mixed path's rounding. */
typedef struct rpa_batch rpa_batch;
int rpa_batch_create(rpa_batch** out, rpa_ctx* parent, int max_q);
int rpa_batch_run(rpa_batch* b, int nq, const rpa_request* reqs, int* status);
/* rpa_batch_run in two halves: launch does the per-request part and launches
 * the graph without waiting for it (reqs, status and the requests' arrays must
 * stay valid until the wait); wait blocks until the graph is done and fills
 * status and the outputs.  Two batches on the same parent can alternate, the
 * per-request part of one overlapping the graph of the other. */
int rpa_batch_launch(rpa_batch* b, int nq, const rpa_request* reqs, int* status);
int rpa_batch_wait(rpa_batch* b);
/* Of the last rpa_batch_run: times4 (may be NULL) = seconds of [0] the
 * per-request part, [1] graph capture and instantiation, [2] the graph's
 * execution, [3] the read-back; the number of grouped launches (tile shapes)
 * and of graph nodes. */
int rpa_batch_info(const rpa_batch* b, double* times4, int* groups, long long* nodes);
const char* rpa_batch_last_error(const rpa_batch* b);
/* Destroys the batch's contexts (before rpa_destroy(parent)). */
int rpa_batch_destroy(rpa_batch* b);

#ifdef __cplusplus
}
#endif

#endif /* RPA_GPU_H */
