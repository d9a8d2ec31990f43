"""ctypes front-end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, always as the checker.  The product library never imports it.

Parity status: unpinned by reference outputs (the reference ships no golden
vectors and its Fortran cannot be compiled in this image); pinned by analytic
known-answer tests and an independent numpy restatement (np_oracle.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "liborc.so")

POL = {"xx": 0, "yy": 1, "zz": 2, "yz": 3, "zy": 4}


class OrcSystem(C.Structure):
    _fields_ = [
        ("ng", C.c_int), ("G", C.c_void_p),
        ("nks", C.c_int), ("nbnd", C.c_int), ("npwx", C.c_int),
        ("npw", C.c_void_p), ("igk", C.c_void_p), ("coeff", C.c_void_p), ("E", C.c_void_p),
        ("R", C.c_void_p), ("RI", C.c_void_p),
        ("ntot", C.c_int), ("ktot", C.c_void_p),
        ("K1", C.c_void_p), ("R1", C.c_void_p), ("K2", C.c_void_p), ("R2", C.c_void_p),
        ("iG0", C.c_void_p),
        ("nlf", C.c_int), ("Glf", C.c_void_p),
        ("q", C.c_double * 3),
    ]


class OrcParams(C.Structure):
    _fields_ = [
        ("ngd", C.c_int), ("nocc", C.c_int), ("no", C.c_int), ("pol", C.c_int),
        ("nthreads", C.c_int), ("nk_list", C.c_int), ("klist", C.c_void_p),
        ("domega", C.c_double), ("eta", C.c_double), ("T", C.c_double), ("Efermi", C.c_double),
        ("lor_cut", C.c_double), ("df_cut", C.c_double), ("Vcell", C.c_double),
        ("Gcar", C.c_double), ("eps", C.c_double),
    ]


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "rpa_oracle.cpp")
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        vp, ip, dp = C.c_void_p, C.c_int, C.c_double
        L.orc_gk_sort.argtypes = [vp, ip, ip, vp, dp, vp, vp, vp]
        L.orc_hpsort_eps.argtypes = [ip, vp, vp, dp]
        L.orc_hpsort_eps.restype = None
        L.orc_occupation.argtypes = [dp, dp, dp, vp, vp]
        L.orc_occupation.restype = None
        L.orc_gfast.argtypes = [vp, vp, ip, vp]
        L.orc_gfast.restype = None
        L.orc_vertex.argtypes = [vp, vp, ip, ip, ip, ip, vp, vp]
        L.orc_sloss_s0.argtypes = [vp, vp, vp]
        L.orc_optabs_s0.argtypes = [vp, vp, vp, vp]
        L.orc_kk_sloss.argtypes = [ip, ip, dp, vp, ip, vp]
        L.orc_kk_sloss.restype = None
        L.orc_kk_optabs.argtypes = [ip, ip, dp, vp, vp]
        L.orc_kk_optabs.restype = None
        L.orc_genV.argtypes = [ip, dp, vp, vp, vp, dp, dp, vp]
        L.orc_genV.restype = None
        L.orc_gjel.argtypes = [vp, ip]
        L.orc_dyson.argtypes = [ip, ip, vp, vp, ip, ip, vp, vp]
        _lib = L
    return _lib


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


class Bound:
    """Holds the Fortran-layout arrays of a synth.System alive for C calls."""

    def __init__(self, s, nthreads: int = 0, klist=None, ngd=None, pol="xx"):
        self.s = s
        self.keep = []

        def k(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            self.keep.append(a)
            return a

        self.G = k(s.G, np.float64)
        self.npw = k(s.npw, np.int32)
        self.igk = k(s.igk, np.int32) if s.igk is not None else None
        self.coeff = k(s.coeff, np.complex128)
        self.E = k(s.E, np.float64)
        self.R = np.asfortranarray(s.R)
        self.RI = np.asfortranarray(s.RI)
        self.keep += [self.R, self.RI]
        self.ktot = k(s.ktot, np.float64)
        self.K1, self.R1 = k(s.K1, np.int32), k(s.R1, np.int32)
        self.K2, self.R2 = k(s.K2, np.int32), k(s.R2, np.int32)
        self.iG0 = k(s.iG0, np.int32)
        self.Glf = k(s.Glf, np.float64)
        self.sys = OrcSystem(
            ng=s.G.shape[0], G=_p(self.G), nks=s.nks, nbnd=s.nbnd, npwx=s.npwx,
            npw=_p(self.npw), igk=_p(self.igk) if self.igk is not None else None,
            coeff=_p(self.coeff), E=_p(self.E), R=_p(self.R), RI=_p(self.RI),
            ntot=s.ntot, ktot=_p(self.ktot), K1=_p(self.K1), R1=_p(self.R1), K2=_p(self.K2),
            R2=_p(self.R2), iG0=_p(self.iG0), nlf=s.nlf, Glf=_p(self.Glf),
            q=(C.c_double * 3)(*[float(x) for x in s.q]))
        self.klist = None
        nk_list = 0
        if klist is not None:
            self.klist = k(np.asarray(klist), np.int32)
            nk_list = self.klist.size
        c = s.cfg
        self.par = OrcParams(
            ngd=int(ngd if ngd is not None else s.ngd), nocc=s.nocc, no=s.no, pol=POL[pol],
            nthreads=nthreads, nk_list=nk_list,
            klist=_p(self.klist) if self.klist is not None else None,
            domega=s.domega, eta=s.eta, T=s.T, Efermi=s.Efermi, lor_cut=c.lor_cut, df_cut=c.df_cut,
            Vcell=s.Vcell, Gcar=s.Gcar, eps=c.eps)

    def refs(self):
        return C.byref(self.sys), C.byref(self.par)


def gfast(b: Bound, ik: int) -> np.ndarray:
    s = b.s
    K1 = int(s.K1[ik])
    nsum = int(s.npw[K1 - 1]) if s.igk is not None else b.par.ngd
    out = np.zeros(s.nlf * nsum, dtype=np.int32)
    lib().orc_gfast(*b.refs(), ik, _p(out))
    return out.reshape(s.nlf, nsum)


def vertex(b: Bound, ik: int, n: int, m: int, current: bool):
    s = b.s
    M = np.zeros(s.nlf, dtype=np.complex128)
    M2 = np.zeros(s.nlf, dtype=np.complex128)
    rc = lib().orc_vertex(*b.refs(), int(current), ik, n, m, _p(M), _p(M2))
    assert rc == 0
    return M, M2


def sloss_s0(b: Bound) -> np.ndarray:
    """Real S0, numpy shape (nlf, nlf, no) == Fortran S0(no, nlf, nlf)."""
    s = b.s
    out = np.zeros((s.nlf, s.nlf, s.no), dtype=np.float64)
    rc = lib().orc_sloss_s0(*b.refs(), _p(out))
    if rc != 0:
        raise RuntimeError("oracle: NGd exceeds a basis size")
    return out


def optabs_s0(b: Bound):
    """Complex S0 (nlf, nlf, 2no+1) == Fortran S0(-no:no, nlf, nlf); Qeff (nlf, nlf) == Qeff(nlf,nlf)^T."""
    s = b.s
    S0 = np.zeros((s.nlf, s.nlf, 2 * s.no + 1), dtype=np.complex128)
    Q = np.zeros((s.nlf, s.nlf), dtype=np.complex128)
    rc = lib().orc_optabs_s0(*b.refs(), _p(S0), _p(Q))
    if rc != 0:
        raise RuntimeError("oracle: NGd exceeds a basis size")
    return S0, Q


def kk_sloss(S0: np.ndarray, domega: float, cmplx_sp: bool = False) -> np.ndarray:
    nlf, _, no = S0.shape
    S0 = np.ascontiguousarray(S0)
    out = np.zeros((nlf, nlf, no - 1), dtype=np.complex128)
    lib().orc_kk_sloss(no, nlf, domega, _p(S0), int(cmplx_sp), _p(out))
    return out


def kk_optabs(S0: np.ndarray, domega: float) -> np.ndarray:
    nlf, _, nw = S0.shape
    no = (nw - 1) // 2
    S0 = np.ascontiguousarray(S0)
    out = np.zeros((nlf, nlf, no - 1), dtype=np.complex128)
    lib().orc_kk_optabs(no, nlf, domega, _p(S0), _p(out))
    return out


def genV(s, c0: float | None = None) -> np.ndarray:
    """Real V, numpy (nlf, nlf) == Fortran V(nlf,nlf)^T."""
    Glf = np.ascontiguousarray(s.Glf, dtype=np.float64)
    parG = np.ascontiguousarray(s.parG, dtype=np.int32)
    q = np.ascontiguousarray(s.q, dtype=np.float64)
    V = np.zeros((s.nlf, s.nlf), dtype=np.float64)
    lib().orc_genV(s.nlf, s.cfg.eps, _p(q), _p(Glf), _p(parG), s.Gcar, float(c0 if c0 else s.c0), _p(V))
    return V


def gjel(a: np.ndarray):
    """In-place Gauss-Jordan inverse of a Fortran-layout square matrix."""
    a = np.asfortranarray(a, dtype=np.complex128).copy(order="F")
    rc = lib().orc_gjel(_p(a), a.shape[0])
    return a, rc


def dyson(chi0: np.ndarray, V: np.ndarray, fast_wt: bool = True, nthreads: int = 0):
    """chi0 numpy (nlf,nlf,no-1) (Fortran chi0(no-1,nlf,nlf)); V numpy (nlf,nlf) (Fortran V)."""
    nlf = chi0.shape[0]
    no = chi0.shape[2] + 1
    chi0 = np.ascontiguousarray(chi0)
    V = np.ascontiguousarray(V)
    WT = np.zeros_like(chi0)
    Ei = np.zeros_like(chi0)
    rc = lib().orc_dyson(no, nlf, _p(chi0), _p(V), int(fast_wt), nthreads, _p(WT), _p(Ei))
    return WT, Ei, rc


def fortran_mat(a_np: np.ndarray) -> np.ndarray:
    """numpy (j,i) reversed-index array -> the matrix with [i,j] indexing."""
    return a_np.T


# ---------------------------------------------------------------------------
# Consumers right after the hot path, restated in Python (small sizes only).
# Arrays use the layout of the other outputs here: (Nlf, Nlf, frequency).

def pi_assembly(chi0: np.ndarray, Qeff: np.ndarray, domega: float, eta_intra: float, c0: float):
    """Optabs calc = 2 (Optabs.f90:575-614), loop for loop: returns
    (Pi_tot(1,1) per io = 1..no-1, sigma (2, no-1) [inter, intra], Pi per io).
    Pi_inter is read inside the (iG, jG) loop, as the driver does, so it holds
    Pi_tot(1,1) with the intraband term once the loop has passed (1,1)."""
    nlf, _, nwo = chi0.shape
    Pi_dia = np.zeros((nlf, nlf), dtype=np.complex128)
    Pi_tot = np.zeros((nlf, nlf), dtype=np.complex128)
    pi11 = np.zeros(nwo, dtype=np.complex128)
    sigma = np.zeros((2, nwo))
    full = np.zeros((nlf, nlf, nwo), dtype=np.complex128)
    for io in range(1, nwo + 1):
        oi = (io - 1) * domega
        Pi_inter = Pi_intra = 0j
        for iG in range(nlf):
            for jG in range(nlf):
                re, im = chi0[iG, jG, io - 1].real, chi0[iG, jG, io - 1].imag
                if io == 1:
                    Pi_dia[iG, jG] = -complex(re, 0.0)
                Pi_tot[iG, jG] = complex(re, im)
                Pi_tot[iG, jG] = Pi_tot[iG, jG] + Pi_dia[iG, jG]
                Pi_inter = Pi_tot[0, 0]
                Pi_intra = Qeff[0, 0] * oi / (oi + 1j * eta_intra)
                Pi_tot[iG, jG] = Pi_tot[iG, jG] + Qeff[iG, jG] * oi / (oi + 1j * eta_intra)
        pi11[io - 1] = Pi_tot[0, 0]
        full[:, :, io - 1] = Pi_tot
        if io > 1:
            sigma[0, io - 1] = (-1j * c0 * Pi_inter / oi).real
            sigma[1, io - 1] = (-1j * c0 * Pi_intra / oi).real
    return pi11, sigma, full


def _w1w2(io: int, no: int, oi: float, domega: float, S: np.ndarray):
    """genW1W2 (Sloss.f90:1062-1171) for all (iG, jG) at once; S[..., jo-1]."""
    W1 = np.zeros(S.shape[:2])
    W2 = np.zeros(S.shape[:2])
    if io == 1:
        for jo in range(2, no + 1):
            oj = (jo - 1) * domega
            fact = domega / oj
            if jo == 2:
                fact = 3.0 / 2.0
            elif jo == no:
                fact = 0.5 * domega / oj
            W1 = W1 - fact * S[..., jo - 1]
        return W1, -W1
    for jo in range(1, no + 1):
        oj = (jo - 1) * domega
        if io == 2:
            if jo != io:
                fact = domega / (oi - oj)
            elif jo == 1:
                fact = 1.0
            elif jo == 2:
                fact = 0.0
            elif jo == 3:
                fact = -3.0 / 2.0
            elif jo == no:
                fact = 0.5 * domega / (oi - oj)
        elif io == no - 1:
            if jo != io:
                fact = domega / (oi - oj)
            elif jo == 1:
                fact = 0.5 * domega / (oi - oj)
            elif jo == no - 2:
                fact = 3.0 / 2.0
            elif jo == no - 1:
                fact = 0.0
            elif jo == no:
                fact = -1.0
        else:
            if jo != io:
                fact = domega / (oi - oj)
            elif jo == 1:
                fact = 0.5 * domega / (oi - oj)
            elif jo == io - 1:
                fact = 3.0 / 2.0
            elif jo == io:
                fact = 0.0
            elif jo == io + 1:
                fact = -3.0 / 2.0
            elif jo == no:
                fact = 0.5 * domega / (oi - oj)
        W1 = W1 + fact * S[..., jo - 1]
        fact = domega / (oi + oj)
        if jo == 1 or jo == no:
            fact = 0.5 * domega / (oi + oj)
        W2 = W2 + fact * S[..., jo - 1]
    return W1, W2


def kk_w(WT: np.ndarray, S0_chi: np.ndarray, V11: float, domega: float):
    """KK transform of W and its self-check (Sloss.f90:486-534): returns
    (Gamma+, Gamma-, [KKS, SKK, 100|KKS/SKK|, Re Gamma(o=0,1,1),
    Re(WT(o=0,1,1) - V(1,1))/2]).  S0_chi: the chi0 spectral function
    (Nlf, Nlf, no); its last row stays in the transform, as in the driver."""
    nlf, _, nwo = WT.shape
    no = nwo + 1
    S = S0_chi.copy()
    S[..., :no - 1] = -(1.0 / np.pi) * WT.imag
    Gp = np.zeros_like(WT)
    Gm = np.zeros_like(WT)
    KKS = SKK = 0.0
    G0 = 0j
    for io in range(1, no):
        oi = (io - 1) * domega
        W1, W2 = _w1w2(io, no, oi, domega, S)
        ImW = -np.pi * S[..., io - 1]
        Gp[..., io - 1] = W1 + 1j * ImW
        Gm[..., io - 1] = -W2 + 0j
        W2KK = W2[0, 0]
        if io == 1:
            G0 = Gp[0, 0, 0]
        Wind = (WT[0, 0, io - 1] - V11).real
        WindKK = Gp[0, 0, io - 1].real - W2KK
        fact = 0.5 * domega if (io == 1 or io == no - 1) else domega
        KKS += fact * (WindKK - Wind) ** 2
        SKK += fact * Wind * Wind
    return Gp, Gm, np.array([KKS, SKK, 100.0 * abs(KKS / SKK), G0.real, (WT[0, 0, 0] - V11).real / 2.0])


# ---------------------------------------------------------------------------
# k-point bookkeeping of the drivers, loop for loop (pure Python; small grids).
# R, RI: Fortran R(48,3,3) as numpy (48, 3, 3) [i, n, m]; k-points (n, 3).

def gen_fbz(kI: np.ndarray, R: np.ndarray, nsym: int, eps: float) -> np.ndarray:
    """genFBZ (Chi_RPA/Optabs.f90:886-933): k(:,jk) = R_i kI_ik for i outer, kept
    when no earlier generated point lies within eps in all components."""
    gen = []
    ktot = []
    for i in range(nsym):
        for ik in range(kI.shape[0]):
            k = [0.0, 0.0, 0.0]
            for n in range(3):
                s = 0.0
                for m in range(3):
                    s = s + float(R[i, n, m]) * float(kI[ik, m])
                k[n] = s
            dup = False
            for lk in gen:
                if abs(k[0] - lk[0]) <= eps and abs(k[1] - lk[1]) <= eps and abs(k[2] - lk[2]) <= eps:
                    dup = True
            gen.append(k)
            if not dup:
                ktot.append(k)
    return np.array(ktot, dtype=np.float64)


def _rot(RI, i, k):
    r = RI[i]
    return [float(r[n, 0]) * k[0] + float(r[n, 1]) * k[1] + float(r[n, 2]) * k[2] for n in range(3)]


def _first_ibz(K, kI, eps):
    for j in range(kI.shape[0]):
        if abs(K[0] - kI[j, 0]) <= eps and abs(K[1] - kI[j, 1]) <= eps and abs(K[2] - kI[j, 2]) <= eps:
            return j
    return -1


def find_k_ibz(ktot: np.ndarray, kI: np.ndarray, RI: np.ndarray, nsym: int, eps: float):
    """findKinIBZ (Chi_RPA/Optabs.f90:776-818) for every FBZ point: (R1, K1)
    1-based; 0 where the reference stops ('Can not find wave vector K')."""
    nki = kI.shape[0]
    R1 = np.zeros(ktot.shape[0], dtype=np.int32)
    K1 = np.zeros_like(R1)
    for ik in range(ktot.shape[0]):
        if ik < nki:
            R1[ik], K1[ik] = 1, ik + 1
            continue
        k = [float(x) for x in ktot[ik]]
        for i in range(1, nsym):
            j = _first_ibz(_rot(RI, i, k), kI, eps)
            if j >= 0:
                R1[ik], K1[ik] = i + 1, j + 1
                break
    return R1, K1


def find_kq(ktot: np.ndarray, kI: np.ndarray, RI: np.ndarray, nsym: int, G: np.ndarray, q, eps: float,
            points=None):
    """findKQinBZ (Chi_RPA/Optabs.f90:820-884) for every FBZ point k and k + q
    (or for the FBZ indices in ``points``): (iG0, R2, K2) 1-based; 0 where the
    reference stops.  The G loop is outer and the FBZ loop inner, as in the
    reference (first match wins)."""
    n = ktot.shape[0]
    out = np.zeros((3, n), dtype=np.int32)
    for ik in (range(n) if points is None else points):
        KQ = [float(ktot[ik, d]) + float(q[d]) for d in range(3)]
        done = False
        for iG in range(G.shape[0]):
            g = G[iG]
            for jk in range(n):
                kt = ktot[jk]
                if (abs(KQ[0] - g[0] - kt[0]) <= eps and abs(KQ[1] - g[1] - kt[1]) <= eps
                        and abs(KQ[2] - g[2] - kt[2]) <= eps):
                    k = [float(x) for x in kt]
                    for i in range(nsym):
                        j = _first_ibz(_rot(RI, i, k), kI, eps)
                        if j >= 0:
                            out[:, ik] = (iG + 1, i + 1, j + 1)
                            done = True
                            break
                    if done:
                        break
            if done:
                break
    return out[0], out[1], out[2]
