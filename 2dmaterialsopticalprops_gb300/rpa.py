"""ctypes binding of librpa_gb300.so (the C ABI of include/rpa_gpu.h).

This is the Python mirror of what the Fortran drivers bind through
ISO_C_BINDING: every call passes the drivers' own Fortran-layout arrays.
The library must be built (``build.build()``); there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librpa_gb300.so")

RPA_OK, RPA_EINVAL, RPA_ENOMEM, RPA_ESINGULAR, RPA_ETIMEOUT, RPA_ECUDA, RPA_ESTATE, RPA_ENOTFOUND = (
    0, -1, -2, -3, -4, -5, -6, -7)
PREC_FP64, PREC_MIXED = 0, 1
MODE_CHARGE, MODE_CURRENT = 0, 1
POL = {"xx": 0, "yy": 1, "zz": 2, "yz": 3, "zy": 4}
KK_OPTABS_COMPLEX, KK_SLOSS_REAL = 1, 2

EXPORTS = ["rpa_create", "rpa_destroy", "rpa_last_error", "rpa_set_gvectors", "rpa_set_symmetry",
           "rpa_load_basis", "rpa_kmap", "rpa_set_q", "rpa_chi0", "rpa_chi0_prefetch", "rpa_kk", "rpa_dyson", "rpa_gfast",
           "rpa_init_igk", "rpa_kk_matrix", "rpa_stage_times", "rpa_chi0_stats", "rpa_accum_tile", "rpa_dyson_noalloc", "rpa_selftest", "rpa_launch_count", "rpa_get_stream", "rpa_synchronize",
           "rpa_basis_info", "rpa_create_shared", "rpa_server_create", "rpa_server_submit", "rpa_server_wait",
           "rpa_server_last_error", "rpa_server_destroy", "rpa_pi", "rpa_kk_w", "rpa_gen_fbz",
           "rpa_find_k_ibz", "rpa_find_kq", "rpa_qe_read_gvectors", "rpa_qe_wfc_info", "rpa_qe_read_wfc",
           "rpa_write_corrfun", "rpa_read_corrfun", "rpa_write_wt", "rpa_autotune",
           "rpa_tune_export", "rpa_tune_import", "rpa_batch_create", "rpa_batch_run", "rpa_batch_info", "rpa_batch_launch", "rpa_batch_wait",
           "rpa_server_create_batched", "rpa_server_batched_count",
           "rpa_batch_last_error", "rpa_batch_destroy"]


class RpaOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("verbose", C.c_int), ("split", C.c_int),
                ("reserved", C.c_int * 4)]


class RpaChi0Args(C.Structure):
    _fields_ = [("mode", C.c_int), ("pol", C.c_int), ("ngd", C.c_int), ("nocc", C.c_int), ("no", C.c_int),
                ("ntot_norm", C.c_int), ("domega", C.c_double), ("eta", C.c_double), ("lor_cut", C.c_double),
                ("df_cut", C.c_double), ("T", C.c_double), ("Efermi", C.c_double), ("Vcell", C.c_double),
                ("Gcar", C.c_double)]


REQ_CHI0, REQ_W = 0, 1


class RpaRequest(C.Structure):
    _fields_ = [("kind", C.c_int), ("kk_variant", C.c_int), ("ntot", C.c_int), ("ktot", C.c_void_p),
                ("K1", C.c_void_p), ("R1", C.c_void_p), ("K2", C.c_void_p), ("R2", C.c_void_p),
                ("iG0", C.c_void_p), ("q", C.c_double * 3), ("nlf", C.c_int), ("ilf", C.c_void_p),
                ("parG", C.c_void_p), ("args", RpaChi0Args), ("c0", C.c_double), ("eps", C.c_double),
                ("S0_out", C.c_void_p), ("Qeff_out", C.c_void_p), ("chi0_out", C.c_void_p),
                ("WT_out", C.c_void_p), ("head_out", C.c_void_p)]


class RpaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"rpa error {code}: {msg}")
        self.code = code


_lib = None


def load_library(path: str = LIB_PATH):
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with 2dmaterialsopticalprops_gb300/build.py")
    L = C.CDLL(path)
    vp, ip, dp = C.c_void_p, C.c_int, C.c_double
    L.rpa_create.argtypes = [C.POINTER(vp), C.POINTER(RpaOpts)]
    L.rpa_destroy.argtypes = [vp]
    L.rpa_last_error.argtypes = [vp]
    L.rpa_last_error.restype = C.c_char_p
    L.rpa_set_gvectors.argtypes = [vp, ip, vp, vp, vp]
    L.rpa_set_symmetry.argtypes = [vp, ip, vp, vp]
    L.rpa_load_basis.argtypes = [vp, ip, ip, ip, vp, vp, vp, vp]
    L.rpa_kmap.argtypes = [vp, ip, vp, vp, vp, vp, vp, vp]
    L.rpa_set_q.argtypes = [vp, vp, ip, vp, vp]
    L.rpa_chi0.argtypes = [vp, C.POINTER(RpaChi0Args), vp, vp]
    L.rpa_chi0_prefetch.argtypes = [vp, ip]
    L.rpa_kk.argtypes = [vp, ip, vp]
    L.rpa_dyson.argtypes = [vp, dp, dp, vp, vp, vp]
    L.rpa_gfast.argtypes = [vp, ip, ip, vp]
    L.rpa_init_igk.argtypes = [ip, vp, ip, ip, vp, dp, vp, vp]
    L.rpa_kk_matrix.argtypes = [ip, ip, dp, vp]
    L.rpa_stage_times.argtypes = [vp, vp]
    L.rpa_chi0_stats.argtypes = [vp, vp]
    L.rpa_accum_tile.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.rpa_dyson_noalloc.argtypes = [vp, vp, ip, ip, vp, vp, vp, C.POINTER(C.c_int)]
    L.rpa_selftest.argtypes = [ip, C.POINTER(C.c_double)]
    L.rpa_launch_count.argtypes = [vp, C.POINTER(C.c_longlong)]
    L.rpa_get_stream.argtypes = [vp, C.POINTER(vp)]
    L.rpa_synchronize.argtypes = [vp]
    L.rpa_basis_info.argtypes = [vp, vp]
    L.rpa_pi.argtypes = [vp, dp, dp, vp, vp, vp]
    L.rpa_kk_w.argtypes = [vp, vp, vp, vp]
    L.rpa_gen_fbz.argtypes = [vp, ip, vp, dp, ip, vp, vp]
    L.rpa_find_k_ibz.argtypes = [vp, ip, vp, ip, vp, dp, vp, vp]
    L.rpa_find_kq.argtypes = [vp, ip, vp, ip, vp, vp, dp, vp, vp, vp]
    cp = C.c_char_p
    L.rpa_qe_read_gvectors.argtypes = [cp, vp, ip, vp, vp, vp, vp]
    L.rpa_qe_wfc_info.argtypes = [cp, ip, vp, vp, vp, vp]
    L.rpa_qe_read_wfc.argtypes = [cp, ip, ip, ip, vp, vp]
    L.rpa_write_corrfun.argtypes = [cp, cp, ip, ip, dp, vp, vp]
    L.rpa_read_corrfun.argtypes = [cp, cp, ip, ip, vp, vp]
    L.rpa_write_wt.argtypes = [cp, ip, ip, dp, vp]
    L.rpa_autotune.argtypes = [vp, C.POINTER(RpaChi0Args), vp]
    L.rpa_tune_export.argtypes = [vp, vp, ip, vp]
    L.rpa_tune_import.argtypes = [vp, cp]
    L.rpa_create_shared.argtypes = [C.POINTER(vp), vp, ip]
    L.rpa_server_create.argtypes = [C.POINTER(vp), vp, ip, dp]
    L.rpa_server_submit.argtypes = [vp, C.POINTER(RpaRequest), C.POINTER(C.c_longlong)]
    L.rpa_server_wait.argtypes = [vp, C.c_longlong, vp]
    L.rpa_server_last_error.argtypes = [vp]
    L.rpa_server_destroy.argtypes = [vp]
    L.rpa_batch_create.argtypes = [C.POINTER(vp), vp, ip]
    L.rpa_server_create_batched.argtypes = [C.POINTER(vp), vp, ip, dp, ip]
    L.rpa_server_batched_count.argtypes = [vp, C.POINTER(C.c_longlong)]
    L.rpa_batch_run.argtypes = [vp, ip, vp, vp]
    L.rpa_batch_launch.argtypes = [vp, ip, vp, vp]
    L.rpa_batch_wait.argtypes = [vp]
    L.rpa_batch_info.argtypes = [vp, vp, C.POINTER(ip), C.POINTER(C.c_longlong)]
    L.rpa_batch_last_error.argtypes = [vp]
    L.rpa_batch_destroy.argtypes = [vp]
    for name in EXPORTS:
        if name in ("rpa_server_last_error", "rpa_batch_last_error"):
            getattr(L, name).restype = C.c_char_p
            continue
        if name != "rpa_last_error":
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def _check_out(a, shape, dtype, name):
    if a.shape != tuple(shape) or a.dtype != dtype or not a.flags.c_contiguous or not a.flags.writeable:
        raise ValueError(f"{name}: out must be a writeable contiguous {np.dtype(dtype).name} array of shape {shape}")


def _p(a):
    return None if a is None else a.ctypes.data


def init_igk(xk: np.ndarray, g: np.ndarray, gcutw: float, npwx: int):
    """init_igk (Modules/qe_gksort.f90:11-42) through the library's host code.

    xk (nks,3), g (ngm,3) in 2pi/alat units.  Returns (igk (nks,npwx), ngk (nks,))."""
    L = load_library()
    xk = np.ascontiguousarray(xk, dtype=np.float64)
    g = np.ascontiguousarray(g, dtype=np.float64)
    nks = xk.shape[0]
    igk = np.zeros((nks, npwx), dtype=np.int32)
    ngk = np.zeros(nks, dtype=np.int32)
    rc = L.rpa_init_igk(nks, _p(xk), npwx, g.shape[0], _p(g), float(gcutw), _p(igk), _p(ngk))
    if rc != RPA_OK:
        raise RpaError(rc, "init_igk: npwx too small or G list too short")
    return igk, ngk


def kk_matrix(variant: int, no: int, domega: float) -> np.ndarray:
    """The KK kernel matrix rpa_kk applies (host code, no device needed)."""
    L = load_library()
    nw = no if variant == KK_SLOSS_REAL else 2 * no + 1
    K = np.zeros((no - 1, nw), dtype=np.float64)
    rc = L.rpa_kk_matrix(variant, no, float(domega), _p(K))
    if rc != RPA_OK:
        raise RpaError(rc, "rpa_kk_matrix: bad arguments")
    return K


def selftest(which: int) -> float:
    """Runs the on-device tcgen05 GEMM self-test; returns its max relative error."""
    L = load_library()
    r = C.c_double()
    rc = L.rpa_selftest(which, C.byref(r))
    if rc != RPA_OK:
        raise RpaError(rc, "rpa_selftest failed")
    return r.value


# -- on-disk formats (host only) ------------------------------------------------
def _io_chk(L, rc):
    if rc != RPA_OK:
        raise RpaError(rc, L.rpa_last_error(None).decode())


def qe_read_gvectors(savedir: str, KC, max_ng: int = 1 << 22):
    """charge-density.dat of a QE 6 save directory: (miller (ng,3), G (ng,3), parG (ng,))."""
    L = load_library()
    KC = np.asfortranarray(KC, dtype=np.float64)
    mil = np.zeros((max_ng, 3), dtype=np.int32)
    G = np.zeros((max_ng, 3))
    par = np.zeros(max_ng, dtype=np.int32)
    ng = C.c_int()
    _io_chk(L, L.rpa_qe_read_gvectors(savedir.encode(), _p(KC), max_ng, C.byref(ng), _p(mil), _p(G), _p(par)))
    n = ng.value
    return mil[:n].copy(), G[:n].copy(), par[:n].copy()


def qe_read_wfc(savedir: str, ik: int, npwx: int | None = None, nbnd: int | None = None):
    """wfc<ik>.dat (1-based ik): (coeff (nbnd, npwx) complex, miller (igwx, 3), xk (3,))."""
    L = load_library()
    igwx, npol, nb = C.c_int(), C.c_int(), C.c_int()
    xk = np.zeros(3)
    _io_chk(L, L.rpa_qe_wfc_info(savedir.encode(), ik, C.byref(igwx), C.byref(npol), C.byref(nb), _p(xk)))
    npwx = npwx or igwx.value
    nbnd = nbnd or nb.value
    coeff = np.zeros((nbnd, npwx), dtype=np.complex128)
    mil = np.zeros((igwx.value, 3), dtype=np.int32)
    _io_chk(L, L.rpa_qe_read_wfc(savedir.encode(), ik, npwx, nbnd, _p(coeff), _p(mil)))
    return coeff, mil, xk


def write_corrfun(path_s0: str, path_qeff: str | None, S0, Qeff, domega: float):
    """S0 and Qeff as Context.chi0 returns them for MODE_CURRENT (their memory is
    Fortran S0(-no:no,nlf,nlf) and Qeff(nlf,nlf))."""
    L = load_library()
    S0 = np.ascontiguousarray(S0, dtype=np.complex128)
    nlf, no = S0.shape[0], (S0.shape[2] - 1) // 2
    Qeff = None if Qeff is None else np.ascontiguousarray(Qeff, dtype=np.complex128)
    _io_chk(L, L.rpa_write_corrfun(path_s0.encode(), None if path_qeff is None else path_qeff.encode(), no, nlf,
                                   domega, _p(S0), _p(Qeff)))


def read_corrfun(path_s0: str, path_qeff: str | None, no: int, nlf: int):
    """The files of write_corrfun (or of the reference's calc = 1): (S0, Qeff)
    in Context.chi0's layout; Qeff None without path_qeff."""
    L = load_library()
    S0 = np.zeros((nlf, nlf, 2 * no + 1), dtype=np.complex128)
    Qeff = np.zeros((nlf, nlf), dtype=np.complex128) if path_qeff else None
    _io_chk(L, L.rpa_read_corrfun(path_s0.encode(), None if path_qeff is None else path_qeff.encode(), no, nlf,
                                  _p(S0), _p(Qeff)))
    return S0, Qeff


def write_wt(path: str, WT, domega: float):
    """WT as Context.dyson returns it (memory = Fortran WT(nw,nlf,nlf))."""
    L = load_library()
    WT = np.ascontiguousarray(WT, dtype=np.complex128)
    _io_chk(L, L.rpa_write_wt(path.encode(), WT.shape[2], WT.shape[0], domega, _p(WT)))


class Context:
    """One rpa_ctx: resident basis + per-q state, Fortran-layout I/O."""

    def __init__(self, device: int = 0, precision: int = PREC_FP64, verbose: int = 0, split: int = 0,
                 tc_seg: int = 0, vertex_simt: bool = False, acc_tile: tuple | None = None):
        self.L = load_library()
        self.h = C.c_void_p()
        opts = RpaOpts(device=device, precision=precision, verbose=verbose, split=split)
        opts.reserved[0] = tc_seg
        # mixed-path vertices: the tensor-core kernel (default) or, chosen
        # explicitly, the FP32 CUDA-core kernel (bases beyond 32767 plane waves
        # or 181 bands per k-point)
        opts.reserved[1] = 1 if vertex_simt else 0
        # mixed-path S0 accumulation tile (gb local fields per G-tile, nio
        # frequency rows per CTA) for every call with M2 = M; None: the
        # autotuner's table, else the library's cost model
        if acc_tile is not None:
            opts.reserved[2] = int(acc_tile[0]) | (int(acc_tile[1]) << 8)
        rc = self.L.rpa_create(C.byref(self.h), C.byref(opts))
        if rc != RPA_OK:
            raise RpaError(rc, self.L.rpa_last_error(None).decode())
        self.precision = precision
        self.nlf = 0
        self.no = 0
        self.mode = None

    def _chk(self, rc: int):
        if rc != RPA_OK:
            raise RpaError(rc, self.L.rpa_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.L.rpa_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- setup ---------------------------------------------------------------
    def set_gvectors(self, miller, G, KC):
        mil = np.ascontiguousarray(miller, dtype=np.int32)
        G = np.ascontiguousarray(G, dtype=np.float64)
        KC = np.asfortranarray(KC, dtype=np.float64)
        self._chk(self.L.rpa_set_gvectors(self.h, mil.shape[0], _p(mil), _p(G), _p(KC)))

    def set_symmetry(self, nsym, R, RI):
        R = np.asfortranarray(R, dtype=np.float64)
        RI = np.asfortranarray(RI, dtype=np.float64)
        self._chk(self.L.rpa_set_symmetry(self.h, nsym, _p(R), _p(RI)))

    # -- k-point bookkeeping (genFBZ, findKinIBZ, findKQinBZ) on the device -----
    def gen_fbz(self, kI, eps: float = 1e-4, max_ntot: int | None = None) -> np.ndarray:
        """FBZ points R_i kI_j (i outer) without eps-duplicates: (ntot, 3)."""
        kI = np.ascontiguousarray(kI, dtype=np.float64)
        cap = max_ntot or 48 * kI.shape[0]
        out = np.zeros((cap, 3))
        n = C.c_int()
        self._chk(self.L.rpa_gen_fbz(self.h, kI.shape[0], _p(kI), eps, cap, C.byref(n), _p(out)))
        return out[:n.value].copy()

    def find_k_ibz(self, ktot, kI, eps: float = 1e-4):
        """(R1, K1), 1-based, for every FBZ point."""
        ktot = np.ascontiguousarray(ktot, dtype=np.float64)
        kI = np.ascontiguousarray(kI, dtype=np.float64)
        R1 = np.zeros(ktot.shape[0], dtype=np.int32)
        K1 = np.zeros_like(R1)
        self._chk(self.L.rpa_find_k_ibz(self.h, ktot.shape[0], _p(ktot), kI.shape[0], _p(kI), eps, _p(R1), _p(K1)))
        return R1, K1

    def find_kq(self, ktot, kI, q, eps: float = 1e-4):
        """(iG0, R2, K2), 1-based, for every FBZ point k and k + q."""
        ktot = np.ascontiguousarray(ktot, dtype=np.float64)
        kI = np.ascontiguousarray(kI, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        n = ktot.shape[0]
        iG0, R2, K2 = (np.zeros(n, dtype=np.int32) for _ in range(3))
        self._chk(self.L.rpa_find_kq(self.h, n, _p(ktot), kI.shape[0], _p(kI), _p(q), eps, _p(iG0), _p(R2), _p(K2)))
        return iG0, R2, K2

    def load_basis(self, npw, igk, coeff, E):
        """npw (nks,), igk (nks,npwx) 1-based or None, coeff (nks,nbnd,npwx) complex, E (nbnd,nks) Ha."""
        npw = np.ascontiguousarray(npw, dtype=np.int32)
        coeff = np.ascontiguousarray(coeff, dtype=np.complex128)
        nks, nbnd, npwx = coeff.shape
        igk_a = None if igk is None else np.ascontiguousarray(igk, dtype=np.int32)
        E = np.ascontiguousarray(E, dtype=np.float64)
        self._chk(self.L.rpa_load_basis(self.h, nks, nbnd, npwx, _p(npw), _p(igk_a), _p(coeff), _p(E)))

    def kmap(self, ktot, K1, R1, K2, R2, iG0):
        ktot = np.ascontiguousarray(ktot, dtype=np.float64)
        arrs = [np.ascontiguousarray(x, dtype=np.int32) for x in (K1, R1, K2, R2, iG0)]
        self._chk(self.L.rpa_kmap(self.h, ktot.shape[0], _p(ktot), *[_p(a) for a in arrs]))

    def set_q(self, q, ilf, parG=None):
        q = np.ascontiguousarray(q, dtype=np.float64)
        ilf = np.ascontiguousarray(ilf, dtype=np.int32)
        par = None if parG is None else np.ascontiguousarray(parG, dtype=np.int32)
        self._chk(self.L.rpa_set_q(self.h, _p(q), ilf.size, _p(ilf), _p(par)))
        self.nlf = ilf.size

    def load_system(self, s):
        """All setup calls for a synth.System (what a driver does before its q loop)."""
        self.set_gvectors(s.miller, s.G, s.KC)
        self.load_basis(s.npw, s.igk, s.coeff, s.E)
        self.kmap(s.ktot, s.K1, s.R1, s.K2, s.R2, s.iG0)
        self.set_q(s.q, s.ilf, s.parG)
        self.sys = s

    # -- the hot path ----------------------------------------------------------
    def chi0(self, mode: int, *, no: int, domega: float, eta: float, Vcell: float, Gcar: float, pol: str = "xx",
             ngd: int = 0, nocc: int = 0, lor_cut: float = 1e-3, df_cut: float = 1e-4, T: float = 0.0,
             Efermi: float = 0.0, ntot_norm: int = 0, want: bool = True, out: tuple | None = None):
        """S0 (and Qeff for the current mode) in the drivers' layouts.  `out`
        may give caller-owned arrays (S0, Qeff or None) of those shapes, e.g.
        page-locked buffers reused from call to call."""
        args = RpaChi0Args(mode=mode, pol=POL[pol], ngd=ngd, nocc=nocc, no=no, ntot_norm=ntot_norm, domega=domega,
                           eta=eta, lor_cut=lor_cut, df_cut=df_cut, T=T, Efermi=Efermi, Vcell=Vcell, Gcar=Gcar)
        nlf = self.nlf
        S0 = Q = None
        cplx = mode == MODE_CURRENT
        s_shape = (nlf, nlf, 2 * no + 1) if cplx else (nlf, nlf, no)
        s_type = np.complex128 if cplx else np.float64
        if out is not None:
            S0, Q = out
            _check_out(S0, s_shape, s_type, "chi0 S0")
            if cplx and Q is not None:
                _check_out(Q, (nlf, nlf), np.complex128, "chi0 Qeff")
            if not cplx:
                Q = None
        elif want:
            S0 = np.zeros(s_shape, dtype=s_type)
            Q = np.zeros((nlf, nlf), dtype=np.complex128) if cplx else None
        self._chk(self.L.rpa_chi0(self.h, C.byref(args), _p(S0), _p(Q)))
        self.no = no
        self.mode = mode
        return S0, Q

    def chi0_prefetch(self, pol: str | None):
        """The next current-mode chi0 (xx, yy or zz) also computes the vertices
        of `pol` and keeps them for a chi0 of `pol` that directly follows with
        the same arguments (rpa_chi0_prefetch); None cancels."""
        self._chk(self.L.rpa_chi0_prefetch(self.h, -1 if pol is None else POL[pol]))

    def kk(self, variant: int, want: bool = True, out: np.ndarray | None = None):
        """chi0 after the KK transform, (nlf, nlf, no-1) complex; `out` may be a
        caller-owned array of that shape (e.g. page-locked memory)."""
        shape = (self.nlf, self.nlf, self.no - 1)
        if out is not None:
            if out.shape != shape or out.dtype != np.complex128 or not out.flags.c_contiguous:
                raise ValueError("kk: out must be a contiguous complex128 array of shape %s" % (shape,))
        elif want:
            out = np.zeros(shape, dtype=np.complex128)
        self._chk(self.L.rpa_kk(self.h, variant, _p(out)))
        return out

    def dyson(self, c0: float, eps: float, want_wt: bool = True, want_epsinv: bool = False, want_head: bool = True,
              out: tuple | None = None):
        """(WT, eps^-1, eps^-1_00); `out` may give caller-owned arrays
        (WT, eps^-1, head; None for an output not wanted)."""
        n, nw = self.nlf, self.no - 1
        if out is not None:
            WT, Ei, head = out
            for a, shp, name in ((WT, (n, n, nw), "WT"), (Ei, (n, n, nw), "eps^-1"), (head, (nw,), "head")):
                if a is not None:
                    _check_out(a, shp, np.complex128, "dyson " + name)
        else:
            WT = np.zeros((n, n, nw), dtype=np.complex128) if want_wt else None
            Ei = np.zeros((n, n, nw), dtype=np.complex128) if want_epsinv else None
            head = np.zeros(nw, dtype=np.complex128) if want_head else None
        rc = self.L.rpa_dyson(self.h, c0, eps, _p(WT), _p(Ei), _p(head))
        self._chk(rc)
        return WT, Ei, head

    def pi(self, eta_intra: float, c0: float, want_full: bool = False):
        """Optabs calc = 2 assembly: (Pi_11 spectrum, sigma[2, no-1] inter/intra, full Pi or None)."""
        nwo = self.no - 1
        p11 = np.zeros(nwo, dtype=np.complex128)
        full = np.zeros((self.nlf, self.nlf, nwo), dtype=np.complex128) if want_full else None
        sig_c = np.zeros(2 * nwo)
        self._chk(self.L.rpa_pi(self.h, eta_intra, c0, _p(p11), _p(sig_c), _p(full)))
        return p11, sig_c.reshape(nwo, 2).T.copy(), full

    def kk_w(self, want_gamma: bool = True):
        """KK transform of W and its self-check: (Gamma+, Gamma-, check5)."""
        nwo = self.no - 1
        gp = np.zeros((self.nlf, self.nlf, nwo), dtype=np.complex128) if want_gamma else None
        gm = np.zeros((self.nlf, self.nlf, nwo), dtype=np.complex128) if want_gamma else None
        chk = np.zeros(5)
        self._chk(self.L.rpa_kk_w(self.h, _p(gp), _p(gm), _p(chk)))
        return gp, gm, chk

    def gfast(self, ik1: int, ngd: int = 0) -> np.ndarray:
        s = self.sys
        K1 = int(s.K1[ik1 - 1])
        nsum = int(s.npw[K1 - 1]) if s.igk is not None else ngd
        out = np.zeros(self.nlf * nsum, dtype=np.int32)
        self._chk(self.L.rpa_gfast(self.h, ik1, ngd, _p(out)))
        return out.reshape(self.nlf, nsum)

    def stage_times(self):
        out = np.zeros(6)
        self._chk(self.L.rpa_stage_times(self.h, _p(out)))
        return dict(zip(["pairs", "vertices", "accumulate", "kk", "dyson", "copies"], out.tolist()))

    def autotune(self, mode: int, **kw) -> float:
        """rpa_autotune for the chi0 call chi0(mode, **kw) would make; returns the
        best vertex-stage time (ms)."""
        pol = kw.pop("pol", "xx")
        args = RpaChi0Args(mode=mode, pol=POL[pol], ngd=kw.get("ngd", 0), nocc=kw.get("nocc", 0), no=kw["no"],
                           ntot_norm=kw.get("ntot_norm", 0), domega=kw["domega"], eta=kw["eta"],
                           lor_cut=kw.get("lor_cut", 1e-3), df_cut=kw.get("df_cut", 1e-4), T=kw.get("T", 0.0),
                           Efermi=kw.get("Efermi", 0.0), Vcell=kw["Vcell"], Gcar=kw["Gcar"])
        ms = C.c_double()
        self._chk(self.L.rpa_autotune(self.h, C.byref(args), C.byref(ms)))
        return ms.value

    def tune_export(self) -> str:
        n = C.c_int()
        self._chk(self.L.rpa_tune_export(self.h, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        self._chk(self.L.rpa_tune_export(self.h, buf, n.value, C.byref(n)))
        return buf.value.decode()

    def tune_import(self, text: str):
        self._chk(self.L.rpa_tune_import(self.h, text.encode()))

    def accum_tile(self) -> tuple:
        """(gb, nio) of the last mixed-path accumulation, (0, 0) if none."""
        gb, nio = C.c_int(), C.c_int()
        self._chk(self.L.rpa_accum_tile(self.h, C.byref(gb), C.byref(nio)))
        return gb.value, nio.value

    def chi0_stats(self):
        out = np.zeros(4)
        self._chk(self.L.rpa_chi0_stats(self.h, _p(out)))
        return dict(zip(["transitions", "sum_nwin", "vertex_macs", "chunks"], out.tolist()))

    def launch_count(self) -> int:
        n = C.c_longlong()
        self._chk(self.L.rpa_launch_count(self.h, C.byref(n)))
        return int(n.value)

    def stream_handle(self) -> int:
        h = C.c_void_p()
        self._chk(self.L.rpa_get_stream(self.h, C.byref(h)))
        return h.value or 0

    def synchronize(self):
        self._chk(self.L.rpa_synchronize(self.h))


def shared_context(parent: Context, precision: int | None = None) -> Context:
    """A Context that uses parent's resident G list, symmetry and basis
    (rpa_create_shared) with its own q, buffers and stream; precision
    defaults to the parent's."""
    c = Context.__new__(Context)
    c.L = parent.L
    c.h = C.c_void_p()
    prec = -1 if precision is None else precision
    rc = c.L.rpa_create_shared(C.byref(c.h), parent.h, prec)
    if rc != RPA_OK:
        raise RpaError(rc, c.L.rpa_last_error(parent.h).decode())
    c.precision, c.nlf, c.no, c.mode = parent.precision if precision is None else precision, 0, 0, None
    c.sys = getattr(parent, "sys", None)
    return c


def _make_request(*, kind: int, kmap: dict, ilf, parG, args: dict, mode: int, kk_variant: int,
                  c0: float = 0.0, eps: float = 1e-4, want_s0: bool = False, want_chi0: bool = True,
                  want_wt: bool = False, want_head: bool = True):
    """An RpaRequest and the arrays it points to (kept alive by the caller)."""
    keep = {}

    def arr(x, dt):
        a = np.ascontiguousarray(x, dtype=dt)
        keep[id(a)] = a
        return a

    ktot = arr(kmap["ktot"], np.float64)
    ints = [arr(kmap[k], np.int32) for k in ("K1", "R1", "K2", "R2", "iG0")]
    ilf_a = arr(ilf, np.int32)
    par_a = arr(parG, np.int32)
    nlf, no = ilf_a.size, int(args["no"])
    a = dict(args)
    pol = POL[a.pop("pol", "xx")]
    ca = RpaChi0Args(mode=mode, pol=pol, **{k: v for k, v in a.items()})
    outs = {}
    if want_s0:
        outs["S0"] = (np.zeros((nlf, nlf, 2 * no + 1), dtype=np.complex128) if mode == MODE_CURRENT
                      else np.zeros((nlf, nlf, no), dtype=np.float64))
    if want_chi0:
        outs["chi0"] = np.zeros((nlf, nlf, no - 1), dtype=np.complex128)
    if kind == REQ_W and want_wt:
        outs["WT"] = np.zeros((nlf, nlf, no - 1), dtype=np.complex128)
    if kind == REQ_W and want_head:
        outs["head"] = np.zeros(no - 1, dtype=np.complex128)
    r = RpaRequest(kind=kind, kk_variant=kk_variant, ntot=ktot.shape[0], ktot=_p(ktot),
                   K1=_p(ints[0]), R1=_p(ints[1]), K2=_p(ints[2]), R2=_p(ints[3]), iG0=_p(ints[4]),
                   nlf=nlf, ilf=_p(ilf_a), parG=_p(par_a), args=ca, c0=c0, eps=eps,
                   S0_out=_p(outs.get("S0")), Qeff_out=None, chi0_out=_p(outs.get("chi0")),
                   WT_out=_p(outs.get("WT")), head_out=_p(outs.get("head")))
    for i in range(3):
        r.q[i] = float(kmap["q"][i])
    return r, keep, outs


class Batch:
    """rpa_batch: up to max_q W requests per run on shared contexts of parent,
    their S0 accumulations as grouped-tile launches and the conversion, KK and
    Dyson stages of all of them in one CUDA graph."""

    def __init__(self, parent: Context, max_q: int):
        self.L = parent.L
        self.h = C.c_void_p()
        rc = self.L.rpa_batch_create(C.byref(self.h), parent.h, int(max_q))
        if rc != RPA_OK:
            raise RpaError(rc, "rpa_batch_create failed")
        self.max_q = int(max_q)
        self._pending = None

    def run(self, requests: list, want_wt: bool = False):
        """requests: dicts with kmap, ilf, parG, args, c0, eps (W requests).
        Returns a list of (status, {"head": ..., "WT": ...})."""
        self.launch(requests, want_wt)
        return self.wait()

    def launch(self, requests: list, want_wt: bool = False):
        """The per-request part and the graph launch; returns without waiting
        for the graph (wait() collects the results)."""
        built = [_make_request(kind=REQ_W, mode=MODE_CHARGE, kk_variant=KK_SLOSS_REAL, want_chi0=False,
                               want_wt=want_wt, **{k: r[k] for k in ("kmap", "ilf", "parG", "args", "c0", "eps")})
                 for r in requests]
        arr = (RpaRequest * len(built))(*[b[0] for b in built])
        st = np.zeros(len(built), dtype=np.int32)
        rc = self.L.rpa_batch_launch(self.h, len(built), C.cast(arr, C.c_void_p), _p(st))
        if rc != RPA_OK:
            raise RpaError(rc, self.L.rpa_batch_last_error(self.h).decode())
        self._pending = (built, arr, st)

    def wait(self):
        if self._pending is None:
            rc = self.L.rpa_batch_wait(self.h)
            raise RpaError(rc, self.L.rpa_batch_last_error(self.h).decode())
        built, arr, st = self._pending
        self._pending = None
        rc = self.L.rpa_batch_wait(self.h)
        if rc != RPA_OK and not np.any(st != RPA_OK):
            raise RpaError(rc, self.L.rpa_batch_last_error(self.h).decode())
        return [(int(s), b[2]) for s, b in zip(st, built)]

    def info(self) -> dict:
        t = np.zeros(4)
        g = C.c_int()
        n = C.c_longlong()
        self.L.rpa_batch_info(self.h, _p(t), C.byref(g), C.byref(n))
        return {"setup_s": t[0], "capture_s": t[1], "graph_s": t[2], "readback_s": t[3], "groups": g.value,
                "graph_nodes": n.value}

    def last_error(self) -> str:
        return self.L.rpa_batch_last_error(self.h).decode()

    def close(self):
        if self.h:
            self.L.rpa_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """rpa_server: requests of any q, local-field set and frequency grid on
    one resident basis, run by nslots shared contexts with continuous
    batching.  submit() returns an id; wait(id) returns the outputs and
    (latency, queue, service) seconds."""

    def __init__(self, parent: Context, nslots: int, mem_bytes: float, batch_q: int = 0):
        """batch_q > 0: also a batching worker that runs up to batch_q queued W
        requests as one rpa_batch (rpa_server_create_batched)."""
        self.L = parent.L
        self.parent = parent
        self.h = C.c_void_p()
        if batch_q > 0:
            rc = self.L.rpa_server_create_batched(C.byref(self.h), parent.h, nslots, float(mem_bytes), int(batch_q))
        else:
            rc = self.L.rpa_server_create(C.byref(self.h), parent.h, nslots, float(mem_bytes))
        if rc != RPA_OK:
            raise RpaError(rc, "rpa_server_create failed")
        self.live = {}

    def submit(self, *, kind: int, kmap: dict, ilf, parG, args: dict, mode: int, kk_variant: int,
               c0: float = 0.0, eps: float = 1e-4, want_s0: bool = False, want_chi0: bool = True,
               want_wt: bool = False, want_head: bool = True) -> int:
        r, keep, outs = _make_request(kind=kind, kmap=kmap, ilf=ilf, parG=parG, args=args, mode=mode,
                                      kk_variant=kk_variant, c0=c0, eps=eps, want_s0=want_s0, want_chi0=want_chi0,
                                      want_wt=want_wt, want_head=want_head)
        rid = C.c_longlong()
        rc = self.L.rpa_server_submit(self.h, C.byref(r), C.byref(rid))
        if rc != RPA_OK:
            raise RpaError(rc, "rpa_server_submit failed")
        self.live[rid.value] = (keep, outs, r)
        return rid.value

    def batched_count(self) -> int:
        n = C.c_longlong()
        self._chk_srv(self.L.rpa_server_batched_count(self.h, C.byref(n)))
        return n.value

    def _chk_srv(self, rc):
        if rc != RPA_OK:
            raise RpaError(rc, "server")

    def wait(self, rid: int):
        t = np.zeros(3)
        rc = self.L.rpa_server_wait(self.h, rid, _p(t))
        keep, outs, _ = self.live.pop(rid)
        if rc != RPA_OK:
            raise RpaError(rc, self.L.rpa_server_last_error(self.h).decode())
        return outs, tuple(t.tolist())

    def close(self):
        if self.h:
            rc = self.L.rpa_server_destroy(self.h)
            self.h = C.c_void_p()
            if rc != RPA_OK:
                raise RpaError(rc, "rpa_server_destroy failed")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# S0 accumulation tile variants of the mixed path, (gb, nio) as the library
# lists them (opts.reserved[2] in include/rpa_gpu.h); the first is the default
ACC_VARIANTS = {"complex": [(96, 1), (64, 1), (32, 2)],
                "real": [(96, 2), (128, 1), (64, 2), (48, 2), (32, 2)]}


def sloss_args(s) -> dict:
    """rpa_chi0 arguments of the Sloss driver for a synth.System."""
    return dict(no=s.no, domega=s.domega, eta=s.eta, Vcell=s.Vcell, Gcar=s.Gcar, nocc=s.nocc,
                ngd=0 if s.igk is not None else s.ngd)


def optabs_args(s, pol: str = "xx") -> dict:
    """rpa_chi0 arguments of the Optabs driver for a synth.System."""
    c = s.cfg
    return dict(no=s.no, domega=s.domega, eta=s.eta, Vcell=s.Vcell, Gcar=s.Gcar, pol=pol, lor_cut=c.lor_cut,
                df_cut=c.df_cut, T=s.T, Efermi=s.Efermi, ngd=0 if s.igk is not None else s.ngd)


def errstats(a: np.ndarray, b: np.ndarray, floor: float = 1e-3) -> dict:
    """Error of a against the reference b, three ways:
    normwise    max |a - b| / max |b|;
    rms         ||a - b||_2 / ||b||_2;
    element     max and RMS over the elements of |a - b| / |b|, taken where
                |b| >= floor * max |b| (elements below the floor are close to
                zero, where a relative error says nothing about the spectrum)."""
    a = np.asarray(a)
    b = np.asarray(b)
    d = np.abs(a - b)
    mb = float(np.abs(b).max()) if b.size else 0.0
    out = {"normwise": float(d.max() / mb) if mb > 0 else float(d.max(initial=0.0)),
           "rms": float(np.linalg.norm(d) / max(np.linalg.norm(b), 1e-300)), "floor": floor}
    sel = np.abs(b) >= floor * mb
    if mb > 0 and sel.any():
        r = d[sel] / np.abs(b[sel])
        out.update({"elem_max": float(r.max()), "elem_rms": float(np.sqrt(np.mean(r ** 2))),
                    "elem_n": int(sel.sum()), "n": int(b.size)})
    else:
        out.update({"elem_max": None, "elem_rms": None, "elem_n": 0, "n": int(b.size)})
    return out


def relerr(a: np.ndarray, b: np.ndarray) -> tuple[float, float]:
    """(max |a-b| / max |b|, ||a-b||_2 / ||b||_2)."""
    a = np.asarray(a)
    b = np.asarray(b)
    nb = float(np.max(np.abs(b))) if b.size else 0.0
    if nb == 0.0:
        return float(np.max(np.abs(a - b))) if a.size else 0.0, 0.0
    return float(np.max(np.abs(a - b)) / nb), float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
