"""GPU parity: every stage of the FP64 CUDA path against the CPU oracle on the
same seeded inputs, through the C ABI.

Tolerances (normwise max relative error, max|a-b| / max|b|): the FP64 path
differs from the oracle only in summation order, so S0, Qeff and chi0 must
agree to 1e-11 and the Dyson outputs (which amplify by the condition number
of eps) to 1e-9.  Index maps must be bit-identical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-11
TOL_DYSON = 1e-9


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module", params=["igk", "legacy"])
def case(request, synth, rpa, orc):
    s = synth.build(synth.config_small(igk=request.param == "igk"))
    ctx = rpa.Context()
    ctx.load_system(s)
    yield s, ctx, orc.Bound(s)
    ctx.close()


def test_gfast_maps_bit_exact(case, orc):
    s, ctx, b = case
    ngd = 0 if s.igk is not None else s.ngd
    for ik in range(s.ntot):
        assert np.array_equal(ctx.gfast(ik + 1, ngd), orc.gfast(b, ik)), ik


def test_sloss_chain(case, rpa, orc):
    s, ctx, b = case
    S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    So = orc.sloss_s0(b)
    assert rel(S, So) < TOL
    st = ctx.chi0_stats()
    assert st["transitions"] > 0 and st["sum_nwin"] >= st["transitions"]
    chi = ctx.kk(rpa.KK_SLOSS_REAL)
    chio = orc.kk_sloss(So, s.domega)
    assert rel(chi, chio) < TOL
    WT, Ei, head = ctx.dyson(s.c0, s.cfg.eps, want_wt=True, want_epsinv=True, want_head=True)
    WTo, Eio, rc = orc.dyson(chio, orc.genV(s), fast_wt=False)
    assert rc == 0
    assert rel(WT, WTo) < TOL_DYSON
    assert rel(Ei, Eio) < TOL_DYSON
    assert rel(head, Eio[0, 0, :]) < TOL_DYSON


@pytest.mark.parametrize("pol", ["xx", "zz", "yz", "zy"])
def test_optabs_chain(case, rpa, orc, pol):
    s, ctx, _ = case
    b = orc.Bound(s, pol=pol)
    S, Q = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, pol))
    So, Qo = orc.optabs_s0(b)
    assert rel(S, So) < TOL
    assert np.abs(Qo).max() > 0 and rel(Q, Qo) < TOL
    chi = ctx.kk(rpa.KK_OPTABS_COMPLEX)
    assert rel(chi, orc.kk_optabs(So, s.domega)) < TOL


def test_results_stay_on_device_without_host_buffers(case, rpa):
    s, ctx, _ = case
    S1, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    chi1 = ctx.kk(rpa.KK_SLOSS_REAL)
    ctx.chi0(rpa.MODE_CHARGE, want=False, **rpa.sloss_args(s))
    chi2 = ctx.kk(rpa.KK_SLOSS_REAL)
    assert np.array_equal(chi1, chi2)  # deterministic order: bitwise repeatable


def test_edge_sizes(synth, rpa, orc):
    """Smallest frequency grid (no=3: only the io=1 and io=2 KK rows), one
    local field, and a frequency window no transition reaches."""
    for kw in (dict(no=3, nlf=1), dict(no=4, nlf=3), dict(no=9, nlf=5, omax_ev=0.2)):
        s = synth.build(synth.config_small(**kw))
        ctx = rpa.Context()
        ctx.load_system(s)
        b = orc.Bound(s)
        S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
        So = orc.sloss_s0(b)
        if np.abs(So).max() == 0:
            assert np.abs(S).max() == 0
        else:
            assert rel(S, So) < TOL
        chi = ctx.kk(rpa.KK_SLOSS_REAL)
        assert np.allclose(chi, orc.kk_sloss(So, s.domega), rtol=0, atol=TOL * max(np.abs(So).max(), 1e-300))
        Sc, Qc = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s))
        Sco, Qco = orc.optabs_s0(b)
        assert np.allclose(Sc, Sco, rtol=0, atol=TOL * max(np.abs(Sco).max(), 1e-300))
        ctx.close()


def test_grid24_off_grid_q_full(synth, rpa, orc):
    """The 24x24, 8-band, NGloc=19, nw=201 workload with q = 0.01 2pi/a off the
    grid (shifted k+q basis), every stage."""
    s = synth.build(synth.config_grid24())
    ctx = rpa.Context()
    ctx.load_system(s)
    b = orc.Bound(s)
    S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    So = orc.sloss_s0(b)
    assert rel(S, So) < TOL
    chio = orc.kk_sloss(So, s.domega)
    assert rel(ctx.kk(rpa.KK_SLOSS_REAL), chio) < TOL
    WT, _, head = ctx.dyson(s.c0, s.cfg.eps)
    WTo, Eio, rc = orc.dyson(chio, orc.genV(s), fast_wt=True)
    assert rel(WT, WTo) < TOL_DYSON
    assert rel(head, Eio[0, 0, :]) < TOL_DYSON
    for pol in ("xx", "zz"):
        Sc, Qc = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, pol))
        Sco, Qco = orc.optabs_s0(orc.Bound(s, pol=pol))
        assert rel(Sc, Sco) < TOL
        if np.abs(Qco).max() > 0:
            assert rel(Qc, Qco) < TOL
    ctx.close()


def test_bad_arguments_are_errors_not_crashes(synth, rpa):
    s = synth.build(synth.config_small())
    ctx = rpa.Context()
    with pytest.raises(rpa.RpaError) as e:
        ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    assert e.value.code == rpa.RPA_ESTATE
    ctx.load_system(s)
    with pytest.raises(rpa.RpaError) as e:
        ctx.kmap(s.ktot, s.K1, s.R1, s.K2 + 10 ** 6, s.R2, s.iG0)
    assert e.value.code == rpa.RPA_EINVAL
    with pytest.raises(rpa.RpaError) as e:
        ctx.set_q(s.q, np.array([0], dtype=np.int32))
    assert e.value.code == rpa.RPA_EINVAL
    ctx.close()


def test_point_group_system(synth, rpa, orc):
    """C6v: FBZ points are rotated IBZ points (R1 != 1) and K+Q lands on
    rotated ones (R2 != 1), so the Gfast maps and the current factors use the
    symmetry matrices.  Maps bit-exact, S0 / Qeff to 1e-11, W to 1e-9."""
    s = synth.build_symmetric(synth.config_small(nk=6, q_steps=1, npw=60, nlf=7, no=31))
    assert len(set(s.R1.tolist())) > 1 and len(set(s.R2.tolist())) > 1
    ctx = rpa.Context()
    ctx.set_gvectors(s.miller, s.G, s.KC)
    ctx.set_symmetry(s.extra["nsym"], s.R, s.RI)
    ctx.load_basis(s.npw, s.igk, s.coeff, s.E)
    ctx.kmap(s.ktot, s.K1, s.R1, s.K2, s.R2, s.iG0)
    ctx.set_q(s.q, s.ilf, s.parG)
    ctx.sys = s
    b = orc.Bound(s)
    for ik in (0, 9, s.ntot - 1):
        assert (ctx.gfast(ik + 1) == orc.gfast(b, ik)).all()
    S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    So = orc.sloss_s0(b)
    assert rel(S, So) < TOL
    chi = ctx.kk(rpa.KK_SLOSS_REAL)
    WT, _, _ = ctx.dyson(s.c0, s.cfg.eps)
    WTo, _, rc = orc.dyson(orc.kk_sloss(So, s.domega), orc.genV(s), fast_wt=True)
    assert rc == 0 and rel(WT, WTo) < TOL_DYSON
    for pol in ("xx", "yz"):
        Sc, Qc = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, pol))
        Sco, Qco = orc.optabs_s0(orc.Bound(s, pol=pol))
        assert rel(Sc, Sco) < TOL and rel(Qc, Qco) < TOL
    ctx.close()
