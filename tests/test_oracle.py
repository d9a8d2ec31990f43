"""CPU checks of the oracle itself: against the independent numpy restatement
and against analytic known-answer cases (the reference ships no test vectors)."""
import math

import numpy as np
import pytest

from conftest import pkg

HARTREE_EV = 2.0 * 13.6056923


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module", params=[True, False], ids=["igk", "legacy"])
def small(request, synth):
    return synth.build(synth.config_small(igk=request.param))


def test_gfast_float_eps_equals_integer_map(small, orc, npo):
    b = orc.Bound(small)
    for ik in range(small.ntot):
        assert np.array_equal(orc.gfast(b, ik), npo.gfast_int(small, ik)), ik


def test_sloss_s0_matches_numpy(small, orc, npo):
    S = orc.sloss_s0(orc.Bound(small))
    assert np.abs(S).max() > 0
    assert rel(S, npo.sloss_s0(small)) < 1e-13


@pytest.mark.parametrize("pol", ["xx", "zz", "yz", "zy"])
def test_optabs_s0_qeff_matches_numpy(small, orc, npo, pol):
    S, Q = orc.optabs_s0(orc.Bound(small, pol=pol))
    Sn, Qn = npo.optabs_s0(small, pol)
    assert rel(S, Sn) < 1e-13
    assert np.abs(Qn).max() > 0
    assert rel(Q, Qn) < 1e-13


def test_kk_and_dyson_match_numpy(small, orc, npo):
    S = orc.sloss_s0(orc.Bound(small))
    chi = orc.kk_sloss(S, small.domega)
    assert rel(chi, npo.kk_sloss(S, small.domega)) < 1e-13
    So, _ = orc.optabs_s0(orc.Bound(small))
    assert rel(orc.kk_optabs(So, small.domega), npo.kk_optabs(So, small.domega)) < 1e-13
    V = orc.genV(small)
    WT, Ei, rc = orc.dyson(chi, V, fast_wt=False)
    assert rc == 0
    WTn, Ein = npo.dyson(chi, V)
    assert rel(WT, WTn) < 1e-12 and rel(Ei, Ein) < 1e-12
    WTf, _, _ = orc.dyson(chi, V, fast_wt=True)
    assert rel(WTf, WT) < 1e-13


def test_threads_do_not_change_results(small, orc):
    a = orc.sloss_s0(orc.Bound(small, nthreads=1))
    b = orc.sloss_s0(orc.Bound(small, nthreads=4))
    assert rel(b, a) < 1e-14


# --- known-answer tests -------------------------------------------------------

def test_single_transition_is_a_cut_lorentzian(synth, orc):
    """One k-point, two bands: S0 is 2 L(o) Re(M M*)/(pi Ntot Vcell) inside
    |L| >= 1e-3/eta and zero outside (Sloss.f90:407-418)."""
    s = synth.build(synth.SynthConfig(nk=1, nbnd=2, nocc=1, npw=40, nlf=3, no=301, omax_ev=20.0, eta_ev=0.2,
                                      q_frac=0.02, igk=True))
    b = orc.Bound(s)
    S = orc.sloss_s0(b)
    M, _ = orc.vertex(b, 0, 1, 2, False)
    e1, e2 = s.E[0, 0], s.E[1, 1]          # E(K1=1,n=1), E(K2=2,m=2)
    o = np.arange(s.no) * s.domega
    L = s.eta / ((o + e1 - e2) ** 2 + s.eta ** 2)
    w = np.where(L >= 1e-3 / s.eta, 2.0 * L / (math.pi * s.ntot * s.Vcell), 0.0)
    X = np.real(np.outer(M, np.conj(M)))
    expect = X.T[:, :, None] * w[None, None, :]    # numpy (jG, iG, io) layout
    assert np.count_nonzero(w) > 0 and np.count_nonzero(w) < s.no
    assert rel(S, expect) < 1e-14


def test_kk_of_lorentzian_matches_cauchy_transform(orc):
    """genChi0 applied to S(w) = (1/pi) eta/((w-w0)^2+eta^2) approximates
    P int S(w')[1/(w-w') - 1/(w+w')] dw' - i pi S(w); for w0 >> eta the
    negative-frequency pole is far and the result is ~ 1/(w - w0 + i eta)
    - 1/(w + w0)."""
    no, dw, w0, eta = 4001, 0.002, 3.0, 0.1
    w = np.arange(no) * dw
    S = (eta / math.pi) / ((w - w0) ** 2 + eta ** 2)
    chi = orc.kk_sloss(S.reshape(1, 1, no), dw)[0, 0]
    wi = w[:-1]
    exact = 1.0 / (wi - w0 + 1j * eta) - 1.0 / (wi + w0 + 1j * eta)
    sel = (wi > 0.5) & (wi < 5.5)
    err = np.abs(chi[sel] - exact[sel]).max() / np.abs(exact[sel]).max()
    assert err < 3e-2


def test_two_by_two_dyson_by_hand(orc):
    chi0 = np.array([[0.3 + 0.1j, 0.05 - 0.02j], [0.04 + 0.01j, 0.2 + 0.3j]])
    V = np.array([[2.0, 0.5], [0.5, 1.0]])
    eps = np.eye(2) - chi0 @ V
    det = eps[0, 0] * eps[1, 1] - eps[0, 1] * eps[1, 0]
    einv = np.array([[eps[1, 1], -eps[0, 1]], [-eps[1, 0], eps[0, 0]]]) / det
    W = V + V @ (einv @ chi0) @ V
    # oracle layouts: numpy (j,i,io) <-> Fortran (io,i,j)
    c = np.stack([chi0.T, chi0.T], axis=-1)
    WT, Ei, rc = orc.dyson(c, V.T.copy(), fast_wt=False)
    assert rc == 0
    assert np.abs(WT[:, :, 0].T - W).max() < 1e-14 * np.abs(W).max() * 10
    assert np.abs(Ei[:, :, 1].T - einv).max() < 1e-14 * 10


def test_gjel_inverse_and_zero_pivot(orc):
    rng = np.random.default_rng(3)
    for n in (1, 2, 7, 33):
        a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        inv, rc = orc.gjel(a)
        assert rc == 0
        assert np.abs(inv - np.linalg.inv(a)).max() < 1e-10
    # 1x1 zero: the zero pivot is reported and the routine carries on (gjel.f:58-59)
    _, rc = orc.gjel(np.zeros((1, 1), dtype=complex))
    assert rc == 2
    # 3x3 zero: after the NaN pivot no candidate passes `>= big`, the stale
    # pivot column is counted twice and gjel stops (gjel.f:39-42)
    _, rc = orc.gjel(np.zeros((3, 3), dtype=complex))
    assert rc == 1


def test_hpsort_eps_ties_order_by_index(orc):
    import ctypes as C
    L = orc.lib()
    ra = np.array([3.0, 1.0, 2.0, 1.0 + 1e-10, 2.0, 0.5])
    ind = np.zeros(ra.size, dtype=np.int32)
    L.orc_hpsort_eps(ra.size, ra.ctypes.data, ind.ctypes.data, 1e-8)
    assert ind.tolist() == [6, 2, 4, 3, 5, 1]


def test_gk_sort_three_ways(synth, orc, rpa):
    """Oracle restatement, the generator's numpy version and the library's
    host init_igk give identical igk lists."""
    s = synth.build(synth.config_small(nk=4))
    ecut = s.extra["ecutw"]
    kpts = s.extra["kpts"]
    npwx = s.npwx + 8
    igk_lib, ngk_lib = rpa.init_igk(kpts, s.G, ecut, npwx)
    for ik in range(kpts.shape[0]):
        igk = np.zeros(npwx, dtype=np.int32)
        gk = np.zeros(npwx)
        ngk = np.zeros(1, dtype=np.int32)
        rc = orc.lib().orc_gk_sort(kpts[ik].ctypes.data, npwx, s.G.shape[0], np.ascontiguousarray(s.G).ctypes.data,
                                   ecut, ngk.ctypes.data, igk.ctypes.data, gk.ctypes.data)
        assert rc == 0
        n = int(ngk[0])
        ref = synth.gk_sort(kpts[ik], s.G, ecut)
        assert n == ref.size == ngk_lib[ik]
        assert np.array_equal(igk[:n], ref)
        assert np.array_equal(igk_lib[ik, :n], ref)
        assert np.all(np.diff(gk[:n]) >= -1e-8)


def test_fortran_default_kind_cmplx_rounding_is_small(small, orc):
    """Sloss.f90:1050 rounds chi0 to single precision (CMPLX without KIND);
    the oracle keeps FP64.  The difference stays at float32 rounding level."""
    S = orc.sloss_s0(orc.Bound(small))
    a = orc.kk_sloss(S, small.domega, cmplx_sp=False)
    b = orc.kk_sloss(S, small.domega, cmplx_sp=True)
    r = rel(b, a)
    assert 0 < r < 1e-6
