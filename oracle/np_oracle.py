"""Independent vectorised numpy restatement -- TEST INFRASTRUCTURE ONLY.

A second, differently-structured restatement of the same reference formulas
used to cross-check the C++ loop oracle on small cases:

* vertices through integer Miller arithmetic and a dictionary lookup instead
  of the float-eps linear search (Sloss.f90:905-944, vertices.f90:122-168);
* S0 through one einsum per k-point instead of per-transition rank-1 loops
  (Sloss.f90:407-418, Optabs.f90:387-443);
* the KK transforms as dense kernel matrices (Sloss.f90:954-1059,
  Optabs.f90:1112-1318);
* the Dyson step with numpy.linalg.inv in place of gjel (Sloss.f90:452-481).
"""
from __future__ import annotations

import math

import numpy as np

PI = 4.0 * math.atan(1.0)


def _lookup(s, kibz1: int):
    """Miller triple -> 1-based position in the basis of IBZ point kibz1."""
    n = int(s.npw[kibz1 - 1])
    if s.igk is not None:
        gidx = s.igk[kibz1 - 1, :n] - 1
    else:
        gidx = np.arange(n)
    return {tuple(s.miller[g].tolist()): i + 1 for i, g in enumerate(gidx)}, gidx


def gfast_int(s, ik: int, ngd: int | None = None) -> np.ndarray:
    """Integer Gfast for FBZ k (0-based); identity symmetry only."""
    K1, K2, iG0 = int(s.K1[ik]), int(s.K2[ik]), int(s.iG0[ik])
    assert int(s.R1[ik]) == 1 and int(s.R2[ik]) == 1
    _, g1 = _lookup(s, K1)
    if s.igk is None:
        g1 = g1[: (ngd or s.ngd)]
    tab2, _ = _lookup(s, K2)
    NG2 = int(s.npw[K2 - 1])
    m0 = s.miller[iG0 - 1]
    out = np.empty((s.nlf, g1.size), dtype=np.int32)
    for a in range(s.nlf):
        mlf = s.miller[s.ilf[a] - 1]
        tgt = s.miller[g1] + mlf + m0
        out[a] = [tab2.get(tuple(t), NG2 + 1) for t in tgt.tolist()]
    return out


def vertices_k(s, ik: int, current: bool, pol: str = "xx", ngd: int | None = None):
    """All band pairs of FBZ k: M[n,m,G] (and M2 for current vertices)."""
    K1, K2 = int(s.K1[ik]), int(s.K2[ik])
    gf = gfast_int(s, ik, ngd)
    nsum = gf.shape[1]
    NG2 = int(s.npw[K2 - 1])
    C1 = s.coeff[K1 - 1, :, :nsum]                     # (nb, nsum)
    C2 = np.concatenate([s.coeff[K2 - 1, :, :NG2], np.zeros((s.nbnd, 1))], axis=1)
    gidx1 = (s.igk[K1 - 1, :nsum] - 1) if s.igk is not None else np.arange(nsum)
    G1 = s.G[gidx1]                                    # (nsum,3) identity R1
    M = np.zeros((s.nbnd, s.nbnd, s.nlf), dtype=np.complex128)
    M2 = np.zeros_like(M)
    comp = {"xx": (0, 0), "yy": (1, 1), "zz": (2, 2), "yz": (1, 2), "zy": (2, 1)}[pol]
    for a in range(s.nlf):
        C2g = C2[:, gf[a] - 1]                          # (nb, nsum)
        if not current:
            M[:, :, a] = np.conj(C1) @ C2g.T
        else:
            j = (s.q[None, :] + 2.0 * s.ktot[ik][None, :] + s.Glf[a][None, :] + 2.0 * G1) * s.Gcar
            w1 = 0.5 * j[:, comp[0]]
            w2 = 0.5 * j[:, comp[1]]
            M[:, :, a] = (np.conj(C1) * w1[None, :]) @ C2g.T
            M2[:, :, a] = (np.conj(C1) * w2[None, :]) @ C2g.T
    return M, (M2 if current else M)


def occupation(Ei, Ef, T):
    x = (Ei - Ef) / T
    if x < -20:
        return 0.0, 1.0
    if x > 20:
        return x, 0.0
    e = math.exp(x)
    return e, 1.0 / (e + 1.0)


def sloss_s0(s, ngd: int | None = None) -> np.ndarray:
    """numpy (nlf,nlf,no) == Fortran S0(no,nlf,nlf)."""
    no, nlf = s.no, s.nlf
    o = np.arange(no) * s.domega
    S = np.zeros((no, nlf, nlf))
    norm = PI * s.ntot * s.Vcell
    for ik in range(s.ntot):
        K1, K2 = int(s.K1[ik]), int(s.K2[ik])
        M, _ = vertices_k(s, ik, False, ngd=ngd)
        n_idx, m_idx = np.meshgrid(np.arange(s.nocc), np.arange(s.nocc, s.nbnd), indexing="ij")
        n_idx, m_idx = n_idx.ravel(), m_idx.ravel()
        dE = o[None, :] + s.E[n_idx, K1 - 1][:, None] - s.E[m_idx, K2 - 1][:, None]
        L = -s.eta / (dE * dE + s.eta * s.eta)
        W = np.where(np.abs(L) >= 1.0e-3 / s.eta, -2.0 * L / norm, 0.0)   # (t, no)
        Mt = M[n_idx, m_idx]                                              # (t, nlf)
        X = np.einsum("tg,th->tgh", Mt, np.conj(Mt)).real
        S += np.einsum("to,tgh->ogh", W, X)
    return np.transpose(S, (2, 1, 0)).copy()


def optabs_s0(s, pol: str = "xx", ngd: int | None = None):
    no, nlf = s.no, s.nlf
    o = np.arange(-no, no + 1) * s.domega
    S = np.zeros((2 * no + 1, nlf, nlf), dtype=np.complex128)
    Q = np.zeros((nlf, nlf), dtype=np.complex128)
    norm = PI * s.ntot * s.Vcell
    cfg = s.cfg
    for ik in range(s.ntot):
        K1, K2 = int(s.K1[ik]), int(s.K2[ik])
        M, M2 = vertices_k(s, ik, True, pol, ngd=ngd)
        for n in range(s.nbnd):
            e1 = s.E[n, K1 - 1]
            ex1, f1 = occupation(e1, s.Efermi, s.T)
            for m in range(s.nbnd):
                e2 = s.E[m, K2 - 1]
                _, f2 = occupation(e2, s.Efermi, s.T)
                df = f1 - f2
                if not (abs(df) >= cfg.df_cut or n == m):
                    continue
                X = np.outer(M[n, m], np.conj(M2[n, m]))
                if n != m:
                    dE = o + e1 - e2
                    L = s.eta / (dE * dE + s.eta * s.eta)
                    w = np.where(np.abs(L) >= cfg.lor_cut / s.eta, -2.0 * df * L / norm, 0.0)
                    S += w[:, None, None] * X[None]
                elif abs(e1 - s.Efermi) <= 10.0 * s.T:
                    fact = -ex1 / ((ex1 + 1.0) ** 2) / s.T
                    Q += 2.0 * fact * X / (s.ntot * s.Vcell)
    return np.transpose(S, (2, 1, 0)).copy(), Q.T.copy()


def kk_matrix_sloss(no: int, domega: float) -> np.ndarray:
    """K[io-1, jo-1] such that Re chi0(io) = sum_jo K S0(jo) (Sloss.f90:954-1059)."""
    K = np.zeros((no - 1, no))
    oj = np.arange(no) * domega
    for io in range(1, no):
        oi = (io - 1) * domega
        if io == 1:
            w = np.zeros(no)
            w[1:] = domega / oj[1:]
            w[1] = 1.5
            if no > 2:
                w[no - 1] = 0.5 * domega / oj[no - 1]
            K[0] = -2.0 * w
            continue
        d = oi - oj
        wm = np.divide(domega, d, out=np.zeros(no), where=(np.arange(1, no + 1) != io))
        wp = domega / (oi + oj)
        wp[0] *= 0.5
        wp[no - 1] *= 0.5 if no - 1 != 0 else 1.0
        K[io - 1] = wm - wp
    return K


def kk_sloss(S0_np: np.ndarray, domega: float) -> np.ndarray:
    S = np.transpose(S0_np, (2, 1, 0))                 # (no, nlf, nlf) [io,i,j]
    no = S.shape[0]
    K = kk_matrix_sloss(no, domega)
    Re = np.einsum("oj,jab->oab", K, S)
    Im = -PI * S[: no - 1]
    return np.transpose(Re + 1j * Im, (2, 1, 0)).copy()


def kk_matrix_optabs(no: int, domega: float):
    """(Kminus, Kplus): chi0(io) = sum_jo Km S0(jo-1) + Kp S0(-jo+1) (+ the pi term)."""
    Km = np.zeros((no - 1, no))
    Kp = np.zeros((no - 1, no))
    for io in range(1, no):
        oi = (io - 1) * domega
        for jo in range(1, no + 1):
            oj = (jo - 1) * domega
            if io == 1:
                if jo == 1:
                    continue
                f = domega / oj
                if jo == 2:
                    f = 1.5
                elif jo == no:
                    f = 0.5 * domega / oj
                Km[0, jo - 1] = -f
                Kp[0, jo - 1] = f
                continue
            f = domega / (oi - oj) if jo != io else 0.0
            if io == 2:
                rules = [(1, 1.0), (2, 0.0), (3, -1.5), (no, None)]
            elif io == no - 1:
                rules = [(1, None), (no - 2, 1.5), (no - 1, 0.0), (no, -1.0)]
            else:
                rules = [(1, None), (io - 1, 1.5), (io, 0.0), (io + 1, -1.5), (no, None)]
            for jj, val in rules:
                if jo == jj:
                    f = (0.5 * domega / (oi - oj)) if val is None else val
                    break
            Km[io - 1, jo - 1] = f
            fp = domega / (oi + oj)
            if jo == 1 or jo == no:
                fp = 0.5 * domega / (oi + oj)
            Kp[io - 1, jo - 1] = fp
    return Km, Kp


def kk_optabs(S0_np: np.ndarray, domega: float) -> np.ndarray:
    S = np.transpose(S0_np, (2, 1, 0))                 # (2no+1, nlf, nlf), index j+no
    no = (S.shape[0] - 1) // 2
    Km, Kp = kk_matrix_optabs(no, domega)
    pos = S[no: 2 * no]                                # S0(0..no-1)
    neg = S[no::-1][:no]                               # S0(0), S0(-1), ..., S0(-(no-1))
    Re = np.einsum("oj,jab->oab", Km, pos.real) + np.einsum("oj,jab->oab", Kp, neg.real)
    Im = np.einsum("oj,jab->oab", Km, pos.imag) + np.einsum("oj,jab->oab", Kp, neg.imag)
    Re = Re + PI * pos[: no - 1].imag
    Im = Im - PI * pos[: no - 1].real
    return np.transpose(Re + 1j * Im, (2, 1, 0)).copy()


def dyson(chi0_np: np.ndarray, V_np: np.ndarray):
    """Returns WT, eps^-1 with the oracle's numpy layouts."""
    chi0 = np.transpose(chi0_np, (2, 1, 0))            # (nw, i, j)
    V = V_np.T                                         # [i,j]
    nw, n, _ = chi0.shape
    eps = np.eye(n)[None] - chi0 @ V[None]
    Ei = np.linalg.inv(eps)
    chi = Ei @ chi0
    WT = V[None] + V[None] @ chi @ V[None]
    return np.transpose(WT, (2, 1, 0)).copy(), np.transpose(Ei, (2, 1, 0)).copy()
