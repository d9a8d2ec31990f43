"""Seeded synthetic Bloch bases in the layout the RPA drivers hand to the library.

The reference reads Quantum ESPRESSO outputs (gvectors.xml / charge-density.dat
for the G list, one coefficient record per band and k-point, a bands.x energy
file, the reciprocal axes and symmetry block of scf.out).  No QE run exists
here, so this module builds the same arrays from a seeded random model:

* a 2D hexagonal cell (lattice constant ``a_ang``, cell height ``c_ang``),
  reciprocal axes KC in 2pi/a0 units (columns b1, b2, b3 as `loadKC` returns
  them, Chi_RPA/Optabs.f90:652-680);
* the G list: Miller triples inside a density sphere, sorted by |G|^2 with
  G(1) = 0 as `loadG` requires (Optabs.f90:1061-1110);
* per IBZ k-point, the k+G basis ordered by QE's gk_sort (Modules/qe_gksort.f90)
  or, in legacy mode, the first ``npw`` entries of the G list for every k;
* band energies from a nearest-neighbour tight-binding dispersion (hopping
  ``t_eV``) stacked into ``nbnd`` bands around E_F = 0, plus N(0, 0.1 eV)
  offsets;
* coefficients drawn N(0,1) and orthonormalised per k-point (QR);
* the identity point group (Nsym = 1), so the FBZ equals the IBZ grid, and
  the K = R1*K1, K+Q = G0 + R2*K2 bookkeeping computed by integer arithmetic
  on the Monkhorst-Pack grid (commensurate q), or, for q off the grid, a
  second seeded basis at the shifted points k+q, as a QE nscf run would give.

Arrays are kept in NumPy C order with the Fortran index order reversed, so
that ``arr.ctypes.data`` is the Fortran column-major array the drivers pass
(e.g. ``coeff`` has shape (nks, nbnd, npwx) == Fortran C(npwx, nbnd, nks)).
"""
from __future__ import annotations

import concurrent.futures as _cf
import math
import os
from dataclasses import dataclass, field

import numpy as np

HARTREE_EV = 2.0 * 13.6056923  # Optabs.f90:50
BOHR_ANG = 0.5291772  # Optabs.f90:52


@dataclass
class SynthConfig:
    nk: int = 24                 # nk x nk Monkhorst-Pack grid (Gamma centred)
    nbnd: int = 8
    nocc: int = 4
    npw: int = 300               # target coefficients per band
    nlf: int = 19                # local fields
    lf: str = "z"                # 'z': G_par = 0 vectors (genGlf lf='z'); 'xyz': first nlf G vectors
    no: int = 201                # frequencies
    omax_ev: float = 30.0
    eta_ev: float = 0.05
    T_ev: float = 0.025852       # 300 K
    a_ang: float = 2.46
    c_ang: float = 20.0
    t_ev: float = 2.7
    band_gap_step_ev: float = 1.0
    q_frac: float = 0.01         # |q| in 2pi/a0 units along Gamma-M (b1 direction)
    q_steps: int | None = None   # commensurate q = q_steps * b1/nk (overrides q_frac)
    igk: bool = True             # per-k gk_sort basis (False: legacy G-list order)
    ngd: int | None = None       # legacy NGd (defaults to min npw)
    seed: int = 1234
    lor_cut: float = 1.0e-3
    df_cut: float = 1.0e-4
    eps: float = 1.0e-4
    threads: int = 0
    # decaying plane-wave envelope: coefficients scaled by exp(-|k+G|^2 / 2 sigma^2)
    # before orthonormalisation, sigma chosen so that the envelope falls by
    # env_decades decades from k+G = 0 to the wavefunction cutoff (0: flat)
    env_decades: float = 0.0


@dataclass
class System:
    cfg: SynthConfig
    a0: float
    c0: float
    Vcell: float
    Gcar: float
    KC: np.ndarray            # (3,3): KC[:, j] = b_j (2pi/a0 units)
    miller: np.ndarray        # (NG,3) int32
    G: np.ndarray             # (NG,3) float64 == Fortran G(3,NG)
    nks: int
    nbnd: int
    nocc: int
    npwx: int
    npw: np.ndarray           # (nks,) int32
    igk: np.ndarray | None    # (nks,npwx) int32, 1-based == Fortran igk_k(npwx,nks)
    ngd: int
    coeff: np.ndarray         # (nks,nbnd,npwx) complex128 == Fortran C(npwx,nbnd,nks)
    E: np.ndarray             # (nbnd,nks) float64 Hartree == Fortran E(nks,nbnd)
    R: np.ndarray             # (48,3,3) [isym,i,j]
    RI: np.ndarray
    ntot: int
    ktot: np.ndarray          # (ntot,3) == Fortran ktot(3,ntot)
    K1: np.ndarray
    R1: np.ndarray
    K2: np.ndarray
    R2: np.ndarray
    iG0: np.ndarray
    nlf: int
    ilf: np.ndarray           # (nlf,) 1-based G indices of the local fields
    Glf: np.ndarray           # (nlf,3)
    parG: np.ndarray          # (nlf,) +-1, parity of the z Miller index
    q: np.ndarray             # (3,) 2pi/a0 units
    no: int
    domega: float             # Hartree
    eta: float                # Hartree
    T: float                  # Hartree
    Efermi: float             # Hartree
    extra: dict = field(default_factory=dict)

    # Fortran-order views for C callers ---------------------------------
    def R_f(self) -> np.ndarray:
        return np.asfortranarray(self.R)

    def RI_f(self) -> np.ndarray:
        return np.asfortranarray(self.RI)


# ---------------------------------------------------------------------------
def hex_cell(a_ang: float, c_ang: float):
    """Bohr lattice constants, cell volume and reciprocal axes (2pi/a0 units)."""
    a0 = a_ang / BOHR_ANG
    c0 = c_ang / BOHR_ANG
    s3 = math.sqrt(3.0)
    # direct axes in units of a0: a1=(1,0,0), a2=(-1/2,sqrt3/2,0), a3=(0,0,c/a)
    b1 = [1.0, 1.0 / s3, 0.0]
    b2 = [0.0, 2.0 / s3, 0.0]
    b3 = [0.0, 0.0, a0 / c0]
    KC = np.array([b1, b2, b3]).T.copy()
    Vcell = a0 * a0 * (s3 / 2.0) * c0
    return a0, c0, Vcell, KC


def g_list(KC: np.ndarray, gcut2: float):
    """All Miller triples with |G|^2 <= gcut2 ((2pi/a0)^2), sorted by |G|^2.

    Ties are ordered by the Miller triple so the order is deterministic.
    """
    b = KC.T  # rows b1,b2,b3
    # bound each Miller index by |G|/|b_i projected| (generous box)
    binv = np.linalg.inv(KC)
    hmax = [int(math.ceil(math.sqrt(gcut2) * np.linalg.norm(binv[i, :]))) + 1 for i in range(3)]
    h = np.arange(-hmax[0], hmax[0] + 1)
    k = np.arange(-hmax[1], hmax[1] + 1)
    l = np.arange(-hmax[2], hmax[2] + 1)
    H, K, L = np.meshgrid(h, k, l, indexing="ij")
    mil = np.stack([H.ravel(), K.ravel(), L.ravel()], axis=1)
    G = mil @ b
    g2 = np.einsum("ij,ij->i", G, G)
    keep = g2 <= gcut2
    mil, G, g2 = mil[keep], G[keep], g2[keep]
    order = np.lexsort((mil[:, 2], mil[:, 1], mil[:, 0], np.round(g2, 10)))
    mil = mil[order].astype(np.int32)
    return mil, (mil.astype(np.float64) @ b)


def gk_sort(k: np.ndarray, G: np.ndarray, ecut: float, npwx: int | None = None):
    """QE gk_sort (Modules/qe_gksort.f90:44-94): igk (1-based) of |k+G|^2 <= ecut.

    Sorted by |k+G|^2 with values closer than 1e-8 treated as equal and then
    ordered by G index, which is what hpsort_eps yields whenever no chain of
    near-equal values spans more than 1e-8 (checked here).
    """
    eps8 = 1.0e-8
    kg = G + k[None, :]
    q = np.einsum("ij,ij->i", kg, kg)
    q[q <= eps8] = 0.0
    g2 = np.einsum("ij,ij->i", G, G)
    q2x = (math.sqrt(float(k @ k)) + math.sqrt(ecut)) ** 2
    inside = np.nonzero(q <= ecut)[0]
    beyond = np.nonzero((q > ecut) & (g2 > q2x + eps8))[0]
    if beyond.size == 0:
        raise ValueError("G list too short for gk_sort (no early exit)")
    stop = beyond[0]
    idx = inside[inside < stop]
    if npwx is not None and idx.size > npwx:
        raise ValueError("npwx too small")
    qq = q[idx]
    o = np.argsort(qq, kind="stable")
    qs, ids = qq[o], idx[o]
    if qs.size == 0:
        return np.zeros(0, dtype=np.int32)
    # runs of eps-equal values are ordered by G index
    brk = np.empty(qs.size, dtype=bool)
    brk[0] = True
    brk[1:] = np.diff(qs) >= eps8
    starts = np.nonzero(brk)[0]
    if np.any(np.maximum.reduceat(qs, starts) - qs[starts] >= eps8):
        raise ValueError("ambiguous eps chain in gk_sort")
    grp = np.cumsum(brk)
    out = ids[np.lexsort((ids, grp))]
    return (out + 1).astype(np.int32)


def tb_energies(kcart: np.ndarray, nbnd: int, nocc: int, t_ev: float, step_ev: float,
                rng: np.random.Generator) -> np.ndarray:
    """Nearest-neighbour graphene-like |f(k)| stacked into nbnd bands (eV)."""
    a1 = np.array([1.0, 0.0, 0.0])
    a2 = np.array([-0.5, math.sqrt(3.0) / 2.0, 0.0])
    ph1 = 2.0 * math.pi * (kcart @ a1)
    ph2 = 2.0 * math.pi * (kcart @ a2)
    f = np.abs(1.0 + np.exp(1j * ph1) + np.exp(1j * ph2))
    E = np.empty((kcart.shape[0], nbnd))
    for n in range(nbnd):
        if n < nocc:
            E[:, n] = -t_ev * f - (nocc - 1 - n) * step_ev
        else:
            E[:, n] = t_ev * f + (n - nocc) * step_ev
    E += rng.normal(0.0, 0.1, size=E.shape)
    return E


def _coeff_block(seed_seq: np.random.SeedSequence, nb: int, npw_list, npwx: int, env=None):
    """N(0,1) complex blocks (times the plane-wave envelope env, (nc, npwx), if
    given) orthonormalised by Cholesky-QR (Q = Z L^-H, Z^H Z = L L^H; the band
    mixing keeps each plane wave's envelope)."""
    rng = np.random.default_rng(seed_seq)
    npw_list = np.asarray(npw_list)
    nc = npw_list.size
    z = rng.standard_normal((nc, npwx, nb, 2)).view(np.complex128)[..., 0]
    z[np.arange(npwx)[None, :] >= npw_list[:, None]] = 0.0
    if env is not None:
        z *= env[:, :, None]
    gram = np.conj(np.transpose(z, (0, 2, 1))) @ z
    L = np.linalg.cholesky(gram)
    # Q^H = L^-1 Z^H
    qh = np.linalg.solve(L, np.conj(np.transpose(z, (0, 2, 1))))
    return np.conj(qh)


def make_coefficients(npw: np.ndarray, nbnd: int, npwx: int, seed: int, tag: int, threads: int = 0,
                      only=None, out: np.ndarray | None = None, env: np.ndarray | None = None):
    """Orthonormal N(0,1) coefficient blocks, seeded per chunk of 64 k-points.

    ``only``: IBZ indices (0-based) whose blocks are needed; the chunks holding
    them are generated (with the same values as a full build) and the rest
    stay zero.  ``out``: preallocated (nks, nbnd, npwx) complex array (e.g.
    page-locked host memory).  ``env``: (nks, npwx) plane-wave envelope."""
    nks = npw.size
    chunk = 64
    starts = list(range(0, nks, chunk))
    ss = np.random.SeedSequence([seed, tag]).spawn(len(starts))
    if out is None:
        out = np.zeros((nks, nbnd, npwx), dtype=np.complex128)
    else:
        out[...] = 0.0
    want = None if only is None else set(int(k) // chunk for k in only)
    nth = threads or min(16, os.cpu_count() or 1)
    with _cf.ThreadPoolExecutor(max_workers=nth) as ex:
        futs = {ex.submit(_coeff_block, ss[i], nbnd, npw[s:s + chunk], npwx,
                          None if env is None else env[s:s + chunk]): s for i, s in enumerate(starts)
                if want is None or i in want}
        for fu in _cf.as_completed(futs):
            s = futs[fu]
            blk = fu.result()
            out[s:s + blk.shape[0]] = blk
    return out


def _count_sphere(G: np.ndarray, radius2: float) -> int:
    return int(np.count_nonzero(np.einsum("ij,ij->i", G, G) <= radius2))


def build(cfg: SynthConfig, coeff_only=None, coeff_out: np.ndarray | None = None) -> System:
    """Builds the seeded system.  ``coeff_only``: FBZ k indices (0-based) whose
    K1/K2 coefficient blocks are needed (others left zero, for sampled CPU
    runs); ``coeff_out``: preallocated coefficient array to fill."""
    a0, c0, Vcell, KC = hex_cell(cfg.a_ang, cfg.c_ang)
    Gcar = 2.0 * math.pi / a0
    b = KC.T
    # wavefunction cutoff giving ~npw plane waves; density sphere of radius 2x
    vol_rec = abs(np.linalg.det(KC))
    r = (3.0 * cfg.npw * vol_rec / (4.0 * math.pi)) ** (1.0 / 3.0)
    kmax = 0.75 * np.linalg.norm(b[0])
    _, Gtrial = g_list(KC, (2.0 * r + 2.0 * kmax) ** 2)
    # refine r so the Gamma sphere holds ~npw vectors
    g2s = np.sort(np.einsum("ij,ij->i", Gtrial, Gtrial))
    target = min(cfg.npw, g2s.size) - 1
    ecutw = float(0.5 * (g2s[target] + g2s[min(target + 1, g2s.size - 1)]))
    gcut_rho = (math.sqrt(ecutw) * 2.0 + 2.0 * kmax) ** 2
    miller, G = g_list(KC, gcut_rho)
    NG = G.shape[0]

    # Monkhorst-Pack grid, Gamma centred: k = i/nk b1 + j/nk b2
    nk = cfg.nk
    ii, jj = np.meshgrid(np.arange(nk), np.arange(nk), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()
    kgrid = (ii[:, None] * b[0] + jj[:, None] * b[1]) / nk
    nks_grid = nk * nk

    rng = np.random.default_rng(np.random.SeedSequence([cfg.seed, 7]))
    E_grid = tb_energies(kgrid, cfg.nbnd, cfg.nocc, cfg.t_ev, cfg.band_gap_step_ev, rng)

    # q and the K+Q bookkeeping
    ntot = nks_grid
    ktot = kgrid.copy()
    K1 = np.arange(1, ntot + 1, dtype=np.int32)
    R1 = np.ones(ntot, dtype=np.int32)
    R2 = np.ones(ntot, dtype=np.int32)
    mil_index = {tuple(m): i + 1 for i, m in enumerate(miller.tolist())}
    if cfg.q_steps is not None:
        s = int(cfg.q_steps)
        q = s * b[0] / nk
        i2 = (ii + s) % nk
        g0 = (ii + s) // nk
        K2 = (i2 * nk + jj + 1).astype(np.int32)
        iG0 = np.array([mil_index[(int(g), 0, 0)] for g in g0], dtype=np.int32)
        kpts = kgrid
        E_all = E_grid
        nks = nks_grid
    else:
        q = cfg.q_frac * b[0] / np.linalg.norm(b[0])
        kq = kgrid + q[None, :]
        rng2 = np.random.default_rng(np.random.SeedSequence([cfg.seed, 8]))
        E_kq = tb_energies(kq, cfg.nbnd, cfg.nocc, cfg.t_ev, cfg.band_gap_step_ev, rng2)
        kpts = np.concatenate([kgrid, kq], axis=0)
        E_all = np.concatenate([E_grid, E_kq], axis=0)
        nks = 2 * nks_grid
        K2 = (np.arange(ntot) + nks_grid + 1).astype(np.int32)
        iG0 = np.ones(ntot, dtype=np.int32)

    # per-k basis
    if cfg.igk:
        igks = [gk_sort(kpts[i], G, ecutw) for i in range(nks)]
        npw = np.array([x.size for x in igks], dtype=np.int32)
        npwx = int(npw.max())
        igk = np.zeros((nks, npwx), dtype=np.int32)
        for i, x in enumerate(igks):
            igk[i, :x.size] = x
        ngd = int(npw.min())
    else:
        nleg = _count_sphere(G, ecutw)
        npw = np.full(nks, nleg, dtype=np.int32)
        npwx = nleg
        igk = None
        ngd = int(cfg.ngd or nleg)
    only = None
    if coeff_only is not None:
        ko = np.asarray(coeff_only, dtype=np.int64)
        only = np.unique(np.concatenate([K1[ko] - 1, K2[ko] - 1]))
    if coeff_out is not None and coeff_out.shape != (nks, cfg.nbnd, npwx):
        raise ValueError(f"coeff_out must have shape {(nks, cfg.nbnd, npwx)}")
    env = None
    if cfg.env_decades > 0:
        # |k+G|^2 of every basis plane wave; exp(-x / 2 sigma^2) = 10^-decades at x = ecutw
        inv2s2 = cfg.env_decades * math.log(10.0) / ecutw
        env = np.zeros((nks, npwx))
        for i in range(nks):
            gi = (igk[i, :npw[i]] - 1) if igk is not None else np.arange(npw[i])
            kg = G[gi] + kpts[i][None, :]
            env[i, :npw[i]] = np.exp(-inv2s2 * np.einsum("ij,ij->i", kg, kg))
    coeff = make_coefficients(npw, cfg.nbnd, npwx, cfg.seed, 11, cfg.threads, only=only, out=coeff_out, env=env)

    # local fields (genGlfandParity, Sloss.f90:824-881), in G-list order:
    # lf='z' keeps G_par = 0 vectors, lf='xyz' the first nlf vectors of the list
    if cfg.lf == "z":
        zsel = np.nonzero((miller[:, 0] == 0) & (miller[:, 1] == 0))[0]
    else:
        zsel = np.arange(miller.shape[0])
    if zsel.size < cfg.nlf:
        raise ValueError("not enough G vectors for nlf")
    ilf = (zsel[:cfg.nlf] + 1).astype(np.int32)
    Glf = G[ilf - 1].copy()
    parG = np.where(miller[ilf - 1, 2] % 2 == 0, 1, -1).astype(np.int32)

    R = np.zeros((48, 3, 3))
    R[0] = np.eye(3)
    RI = R.copy()

    omax = cfg.omax_ev / HARTREE_EV
    domega = omax / (cfg.no - 1)
    sysd = System(cfg=cfg, a0=a0, c0=c0, Vcell=Vcell, Gcar=Gcar, KC=KC, miller=miller, G=G,
                  nks=nks, nbnd=cfg.nbnd, nocc=cfg.nocc, npwx=npwx, npw=npw, igk=igk, ngd=ngd,
                  coeff=coeff, E=np.ascontiguousarray((E_all / HARTREE_EV).T), R=R, RI=RI,
                  ntot=ntot, ktot=ktot, K1=K1, R1=R1, K2=K2, R2=R2, iG0=iG0, nlf=cfg.nlf,
                  ilf=ilf, Glf=Glf, parG=parG, q=q, no=cfg.no, domega=domega,
                  eta=cfg.eta_ev / HARTREE_EV, T=cfg.T_ev / HARTREE_EV, Efermi=0.0)
    sysd.extra["ecutw"] = ecutw
    sysd.extra["kpts"] = kpts
    return sysd


def build_symmetric(cfg: SynthConfig) -> System:
    """A seeded system with the C6v point group: bases, coefficients and
    energies live on the IBZ of the Gamma-centred nk x nk grid (mp_ibz); the FBZ
    points are the images R_i kI_j (i outer, first occurrence kept, with R1 / K1
    the generating operation and IBZ point) and K+Q is matched to an FBZ point
    modulo G (iG0), whose R1 / K1 become R2 / K2.  q = q_steps b1 / nk."""
    a0, c0, Vcell, KC = hex_cell(cfg.a_ang, cfg.c_ang)
    Gcar = 2.0 * math.pi / a0
    b = KC.T
    nsym, R, RI = hex_symmetry()
    nk = cfg.nk
    kI = mp_ibz(KC, nk, R, nsym)
    nki = kI.shape[0]
    vol_rec = abs(np.linalg.det(KC))
    r = (3.0 * cfg.npw * vol_rec / (4.0 * math.pi)) ** (1.0 / 3.0)
    kmax = np.linalg.norm(b[0])
    _, Gtrial = g_list(KC, (2.0 * r + 2.0 * kmax) ** 2)
    g2s = np.sort(np.einsum("ij,ij->i", Gtrial, Gtrial))
    target = min(cfg.npw, g2s.size) - 1
    ecutw = float(0.5 * (g2s[target] + g2s[min(target + 1, g2s.size - 1)]))
    miller, G = g_list(KC, (math.sqrt(ecutw) * 2.0 + 2.0 * kmax) ** 2)
    # FBZ: images R_i kI_j, i outer, first occurrence kept
    ktot, K1, R1 = [], [], []
    for i in range(nsym):
        for j in range(nki):
            k = R[i] @ kI[j]
            if all(np.abs(k - kk).max() > 1e-6 for kk in ktot):
                ktot.append(k)
                K1.append(j + 1)
                R1.append(i + 1)
    ktot = np.array(ktot)
    K1 = np.array(K1, dtype=np.int32)
    R1 = np.array(R1, dtype=np.int32)
    ntot = ktot.shape[0]
    # K+Q = G + ktot_jk
    q = (cfg.q_steps or 1) * b[0] / nk
    Kinv = np.linalg.inv(KC)
    mil_index = {tuple(m): i + 1 for i, m in enumerate(miller.tolist())}
    K2 = np.zeros(ntot, dtype=np.int32)
    R2 = np.zeros(ntot, dtype=np.int32)
    iG0 = np.zeros(ntot, dtype=np.int32)
    for ik in range(ntot):
        kq = ktot[ik] + q
        for jk in range(ntot):
            d = Kinv @ (kq - ktot[jk])
            m = np.rint(d)
            if np.abs(d - m).max() < 1e-6 and tuple(int(x) for x in m) in mil_index:
                iG0[ik] = mil_index[tuple(int(x) for x in m)]
                K2[ik], R2[ik] = K1[jk], R1[jk]
                break
        if iG0[ik] == 0:
            raise ValueError("K+Q not on the grid")
    rng = np.random.default_rng(np.random.SeedSequence([cfg.seed, 7]))
    E_ibz = tb_energies(kI, cfg.nbnd, cfg.nocc, cfg.t_ev, cfg.band_gap_step_ev, rng)
    igks = [gk_sort(kI[i], G, ecutw) for i in range(nki)]
    npw = np.array([x.size for x in igks], dtype=np.int32)
    npwx = int(npw.max())
    igk = np.zeros((nki, npwx), dtype=np.int32)
    for i, x in enumerate(igks):
        igk[i, :x.size] = x
    coeff = make_coefficients(npw, cfg.nbnd, npwx, cfg.seed, 11, cfg.threads)
    if cfg.lf == "z":
        zsel = np.nonzero((miller[:, 0] == 0) & (miller[:, 1] == 0))[0]
    else:
        zsel = np.arange(miller.shape[0])
    ilf = (zsel[:cfg.nlf] + 1).astype(np.int32)
    Glf = G[ilf - 1].copy()
    parG = np.where(miller[ilf - 1, 2] % 2 == 0, 1, -1).astype(np.int32)
    omax = cfg.omax_ev / HARTREE_EV
    domega = omax / (cfg.no - 1)
    s = System(cfg=cfg, a0=a0, c0=c0, Vcell=Vcell, Gcar=Gcar, KC=KC, miller=miller, G=G,
               nks=nki, nbnd=cfg.nbnd, nocc=cfg.nocc, npwx=npwx, npw=npw, igk=igk, ngd=int(npw.min()),
               coeff=coeff, E=np.ascontiguousarray((E_ibz / HARTREE_EV).T), R=R, RI=RI,
               ntot=ntot, ktot=ktot, K1=K1, R1=R1, K2=K2, R2=R2, iG0=iG0, nlf=cfg.nlf,
               ilf=ilf, Glf=Glf, parG=parG, q=q, no=cfg.no, domega=domega,
               eta=cfg.eta_ev / HARTREE_EV, T=cfg.T_ev / HARTREE_EV, Efermi=0.0)
    s.extra["ecutw"] = ecutw
    s.extra["kpts"] = kI
    s.extra["nsym"] = nsym
    return s


def q_kmap(s: System, steps: int, steps2: int = 0) -> dict:
    """K+Q bookkeeping of the commensurate q = (steps b1 + steps2 b2) / nk on
    the Gamma-centred grid of a system built with q_steps: the basis is
    unchanged, only K2 and iG0 move.  Returns rpa_kmap / rpa_set_q inputs."""
    nk = s.cfg.nk
    if s.cfg.q_steps is None:
        raise ValueError("q_kmap needs a system on a commensurate grid (q_steps)")
    b = s.KC.T
    ii, jj = np.meshgrid(np.arange(nk), np.arange(nk), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()
    i2, j2 = (ii + steps) % nk, (jj + steps2) % nk
    g1, g2 = (ii + steps) // nk, (jj + steps2) // nk
    mil_index = {tuple(m): i + 1 for i, m in enumerate(s.miller.tolist())}
    return dict(q=(steps * b[0] + steps2 * b[1]) / nk, ktot=s.ktot, K1=s.K1, R1=s.R1, R2=s.R2,
                K2=(i2 * nk + j2 + 1).astype(np.int32),
                iG0=np.array([mil_index[(int(a), int(c), 0)] for a, c in zip(g1, g2)], dtype=np.int32))


def local_fields(s: System, q: np.ndarray, gcut2: float, lf: str = "xyz", nmax: int | None = None):
    """Local fields of a q-point as genGlf chooses them: the G vectors (all, or
    only G_par = 0 for lf='z') with |q + G|^2 <= gcut2 (2pi/a0 units), in
    G-list order, at most nmax.  Returns (ilf 1-based, parG)."""
    qg = s.G + np.asarray(q)[None, :]
    ok = np.einsum("ij,ij->i", qg, qg) <= gcut2
    if lf == "z":
        ok &= (s.miller[:, 0] == 0) & (s.miller[:, 1] == 0)
    sel = np.nonzero(ok)[0]
    if nmax is not None:
        sel = sel[:nmax]
    ilf = (sel + 1).astype(np.int32)
    parG = np.where(s.miller[sel, 2] % 2 == 0, 1, -1).astype(np.int32)
    return ilf, parG


# Point group and irreducible wedge ------------------------------------------
def hex_symmetry():
    """C6v of the hexagonal cell of hex_cell in Cartesian coordinates: the six
    rotations about z, then the six rotation x mirror(y -> -y) products; the
    identity first.  Returns (nsym, R, RI) as (48, 3, 3) arrays (Fortran
    R(48,3,3) layout when passed with order='F')."""
    h = math.sqrt(3.0) / 2.0
    cs = [(1.0, 0.0), (0.5, h), (-0.5, h), (-1.0, 0.0), (-0.5, -h), (0.5, -h)]
    ops = []
    for c, s in cs:
        ops.append(np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]]))
    for c, s in cs:
        ops.append(np.array([[c, s, 0.0], [s, -c, 0.0], [0.0, 0.0, 1.0]]))
    R = np.zeros((48, 3, 3))
    RI = np.zeros((48, 3, 3))
    for i, r in enumerate(ops):
        R[i] = r
        RI[i] = r.T  # orthogonal
    return len(ops), R, RI


def mp_ibz(KC: np.ndarray, nk: int, R: np.ndarray, nsym: int) -> np.ndarray:
    """IBZ of the Gamma-centred nk x nk grid: grid points in order (i outer),
    each kept unless a symmetry image of it is, modulo the reciprocal lattice,
    an already kept point; kept points are folded into the Wigner-Seitz cell.
    (n, 3) Cartesian, 2pi/a0 units.  The operations act on the grid indices as
    integer matrices (crystal coordinates)."""
    b = KC.T
    Kinv = np.linalg.inv(KC)
    Rc = [np.rint(Kinv @ R[s] @ KC).astype(np.int64) for s in range(nsym)]
    seen = np.zeros((nk, nk), dtype=bool)
    shifts = [i * b[0] + j * b[1] for i in (-1, 0, 1) for j in (-1, 0, 1)]
    kept = []
    for i in range(nk):
        for j in range(nk):
            if seen[i, j]:
                continue
            for r in Rc:
                a, c = (r[0, 0] * i + r[0, 1] * j) % nk, (r[1, 0] * i + r[1, 1] * j) % nk
                seen[a, c] = True
            k = (i * b[0] + j * b[1]) / nk
            kept.append(min((k - s for s in shifts), key=lambda v: (round(float(v @ v), 9), tuple(np.round(v, 9)))))
    return np.array(kept)


# Named workloads -------------------------------------------------------------
def config_small(**kw) -> SynthConfig:
    """A few-second oracle case with the C1 shapes scaled down."""
    base = dict(nk=6, nbnd=8, nocc=4, npw=60, nlf=7, no=41, omax_ev=30.0, eta_ev=0.3, q_steps=1)
    base.update(kw)
    return SynthConfig(**base)


def config_grid24(**kw) -> SynthConfig:
    """24x24 grid, 8 bands (4 occupied), 300 coefficients, NGloc=19, nw=201,
    q = 0.01 2pi/a along Gamma-M, eta = 50 meV."""
    base = dict(nk=24, nbnd=8, nocc=4, npw=300, nlf=19, no=201, omax_ev=30.0, eta_ev=0.05, q_frac=0.01)
    base.update(kw)
    return SynthConfig(**base)


def config_grid120(**kw) -> SynthConfig:
    """120x120 grid, 30 bands (8 occupied), 1500 coefficients, NGloc=91,
    nw=1001 on 0-30 eV, eta = 25 meV, q one grid step along Gamma-M."""
    base = dict(nk=120, nbnd=30, nocc=8, npw=1500, nlf=91, no=1001, omax_ev=30.0, eta_ev=0.025, q_steps=1)
    base.update(kw)
    return SynthConfig(**base)
