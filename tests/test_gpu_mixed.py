"""GPU: the mixed-precision path (tcgen05 split-bf16 accumulation) against the
FP64 oracle.

Tolerance: 1e-5 max relative error, the accuracy the mixed path is built to, applied here
normwise (max |a - b| / max |b|) to S0, chi0 and W, and to Im eps^-1_00 (the
loss function) element-wise relative to its maximum."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def ctx_small(synth, rpa):
    s = synth.build(synth.config_small())
    ctx = rpa.Context(precision=rpa.PREC_MIXED)
    ctx.load_system(s)
    yield s, ctx
    ctx.close()


def test_mixed_sloss_s0(ctx_small, rpa, orc):
    s, ctx = ctx_small
    S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    So = orc.sloss_s0(orc.Bound(s))
    assert rel(S, So) < TOL


@pytest.mark.parametrize("pol", ["xx", "yz"])
def test_mixed_optabs_s0(ctx_small, rpa, orc, pol):
    s, ctx = ctx_small
    S, Q = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, pol))
    So, Qo = orc.optabs_s0(orc.Bound(s, pol=pol))
    assert rel(S, So) < TOL
    assert rel(Q, Qo) < TOL


def test_mixed_multi_tile_nlf131(synth, rpa, orc):
    """nlf = 131 spans two 128-row G tiles and two 96-row G' tiles."""
    s = synth.build(synth.config_small(npw=200, nlf=131, lf="xyz", no=21))
    ctx = rpa.Context(precision=rpa.PREC_MIXED)
    ctx.load_system(s)
    for pol in ("xx", "yz"):
        S, _ = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, pol))
        So, _ = orc.optabs_s0(orc.Bound(s, pol=pol))
        assert rel(S, So) < TOL
    S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    assert rel(S, orc.sloss_s0(orc.Bound(s))) < TOL
    ctx.close()


def test_mixed_three_tiles_symmetric_skip(synth, rpa, orc):
    """nlf = 250 spans three 96-row tiles: with M2 = M (xx, charge) only the
    six tile pairs gi <= gj are accumulated and the other three are mirrored
    (conjugated for the complex S0) when S0 is converted to FP64; the yz pair
    (M2 != M) computes all nine."""
    s = synth.build(synth.config_small(npw=300, nlf=250, lf="xyz", no=21))
    ctx = rpa.Context(precision=rpa.PREC_MIXED)
    ctx.load_system(s)
    for pol in ("xx", "yz"):
        S, Q = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, pol))
        So, Qo = orc.optabs_s0(orc.Bound(s, pol=pol))
        assert rel(S, So) < TOL
        assert rel(Q, Qo) < TOL
    S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    assert rel(S, orc.sloss_s0(orc.Bound(s))) < TOL
    ctx.close()


def test_mixed_grid24_loss_function(synth, rpa, orc):
    s = synth.build(synth.config_grid24())
    ctx = rpa.Context(precision=rpa.PREC_MIXED)
    ctx.load_system(s)
    S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    ctx.kk(rpa.KK_SLOSS_REAL, want=False)
    WT, _, head = ctx.dyson(s.c0, s.cfg.eps)
    So = orc.sloss_s0(orc.Bound(s))
    chio = orc.kk_sloss(So, s.domega)
    WTo, Eio, rc = orc.dyson(chio, orc.genV(s), fast_wt=True)
    assert rel(S, So) < TOL
    assert rel(head.imag, Eio[0, 0, :].imag) < TOL
    assert rel(WT, WTo) < TOL
    ctx.close()


def test_bf16_split_variant_runs(synth, rpa, orc):
    """The bf16 hi/lo operand split (opts.split = 1): same kernel, 8 fewer
    mantissa bits per operand half; checked against a looser 1e-4 bound."""
    s = synth.build(synth.config_small())
    ctx = rpa.Context(precision=rpa.PREC_MIXED, split=1)
    ctx.load_system(s)
    S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    assert rel(S, orc.sloss_s0(orc.Bound(s))) < 1e-4
    ctx.close()


@pytest.mark.parametrize("nbnd,nocc", [(80, 13), (40, 20)])
def test_mixed_band_windows_over_32(synth, rpa, orc, nbnd, nocc):
    """More than 32 bands on a side of the vertex GEMM: the tensor-core vertex
    kernel runs once per pair of band windows (80 bands / 13 occupied: 3
    windows of empty bands for the charge vertex; 40 bands: 2 x 2 windows for
    the current vertex)."""
    s = synth.build(synth.config_small(nbnd=nbnd, nocc=nocc, npw=160, nlf=9, no=31))
    ctx = rpa.Context(precision=rpa.PREC_MIXED)
    ctx.load_system(s)
    S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    assert rel(S, orc.sloss_s0(orc.Bound(s))) < TOL
    Sc, _ = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, "zz"))
    Sco, _ = orc.optabs_s0(orc.Bound(s, pol="zz"))
    assert rel(Sc, Sco) < TOL
    ctx.close()


def test_mixed_legacy_basis(synth, rpa, orc):
    """A basis without an igk map (legacy drivers, NGd coefficients summed): the
    charge vertices gather the empty bands through Gfast (no inverse map)."""
    s = synth.build(synth.config_small(igk=False))
    ctx = rpa.Context(precision=rpa.PREC_MIXED)
    ctx.load_system(s)
    S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    assert rel(S, orc.sloss_s0(orc.Bound(s))) < TOL
    Sc, Qc = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, "yz"))
    Sco, Qco = orc.optabs_s0(orc.Bound(s, pol="yz"))
    assert rel(Sc, Sco) < TOL
    assert rel(Qc, Qco) < TOL
    ctx.close()


def test_vertex_kernels_agree(synth, rpa, orc):
    """The MN-major vertex kernel (default), the K-major tensor-core kernel and
    the FP32 CUDA-core kernel give the same S0 to the mixed-path tolerance."""
    s = synth.build(synth.config_small(nbnd=12, nocc=3, npw=120, nlf=11, no=31))
    ref = rpa.Context(precision=rpa.PREC_MIXED)
    alt = rpa.Context(precision=rpa.PREC_MIXED, vertex_simt=True)
    for c in (ref, alt):
        c.load_system(s)
    So = orc.sloss_s0(orc.Bound(s))
    a, _ = ref.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    b, _ = alt.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    assert rel(a, So) < TOL and rel(b, So) < TOL
    Sco, _ = orc.optabs_s0(orc.Bound(s, pol="xx"))
    a, _ = ref.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, "xx"))
    b, _ = alt.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, "xx"))
    assert rel(a, Sco) < TOL and rel(b, Sco) < TOL
    ref.close()
    alt.close()


@pytest.mark.parametrize("nbnd,nocc,nlf", [(30, 8, 11), (40, 12, 8)])
def test_current_vertices_32_band_windows(synth, rpa, orc, nbnd, nocc, nlf):
    """Current vertices in 32-band windows (one window, and two windows on
    each side), odd NGloc, plane-wave counts that are not a multiple of the
    32-plane-wave chunk: S0 and Qeff of xx, zz and the yz pair against the
    oracle, then xx with zz prefetched (the two-component pass in every pair
    of band windows)."""
    s = synth.build(synth.config_small(nbnd=nbnd, nocc=nocc, npw=150, nlf=nlf, no=31))
    ctx = rpa.Context(precision=rpa.PREC_MIXED)
    ctx.load_system(s)
    ref = {}
    for pol in ("xx", "zz", "yz"):
        So, Qo = orc.optabs_s0(orc.Bound(s, pol=pol))
        ref[pol] = (So, Qo)
        a, qa = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, pol))
        assert rel(a, So) < TOL
        assert rel(qa, Qo) < TOL
    ctx.chi0_prefetch("zz")
    for pol in ("xx", "zz"):
        a, qa = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, pol))
        assert rel(a, ref[pol][0]) < TOL and rel(qa, ref[pol][1]) < TOL, pol
    ctx.close()


def test_autotune_and_every_vertex_configuration(synth, rpa, orc):
    """rpa_autotune keeps one configuration per shape; every configuration it can
    choose (band-window width, gathered side) gives S0 within the mixed-path
    tolerance, and the table survives an export / import round trip."""
    import json
    s = synth.build(synth.config_small(nbnd=24, nocc=5, npw=120, nlf=11, no=31))
    ctx = rpa.Context(precision=rpa.PREC_MIXED)
    ctx.load_system(s)
    So = orc.sloss_s0(orc.Bound(s))
    Sco, _ = orc.optabs_s0(orc.Bound(s, pol="zz"))
    ms = ctx.autotune(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    assert ms > 0
    ctx.autotune(rpa.MODE_CURRENT, **rpa.optabs_args(s, "zz"))
    table = json.loads(ctx.tune_export())["vertex"]
    assert {e["mode"] for e in table} == {rpa.MODE_CHARGE, rpa.MODE_CURRENT}
    S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    assert rel(S, So) < TOL
    nlf32 = s.nlf // 32
    for ymax in (16, 32, 48, 64):
        for swap in (0, 1):
            ctx.tune_import(json.dumps({"vertex": [{"mode": rpa.MODE_CHARGE, "nbnd": 24, "nocc": 5, "nlf32": nlf32,
                                                    "ymax": ymax, "swap": swap}]}))
            S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
            assert rel(S, So) < TOL, (ymax, swap)
    for ymax in (16, 32):
        ctx.tune_import(json.dumps({"vertex": [{"mode": rpa.MODE_CURRENT, "nbnd": 24, "nocc": 0, "nlf32": nlf32,
                                                "ymax": ymax, "swap": -1}]}))
        S, _ = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, "zz"))
        assert rel(S, Sco) < TOL, ymax
    other = rpa.Context(precision=rpa.PREC_MIXED)
    other.tune_import(json.dumps({"vertex": table}))
    assert json.loads(other.tune_export())["vertex"] == table
    with pytest.raises(rpa.RpaError):
        other.tune_import('{"vertex": [{"mode": 0, "nbnd": 24, "nocc": 5, "nlf32": 0, "ymax": 24, "swap": 1}]}')
    fp = rpa.Context()
    fp.load_system(s)
    with pytest.raises(rpa.RpaError) as e:
        fp.autotune(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    assert e.value.code == rpa.RPA_ESTATE
    for c in (ctx, other, fp):
        c.close()


def test_mixed_point_group_system(synth, rpa, orc):
    """The tensor-core vertices with symmetry operations in the maps (C6v):
    both gathered sides of the charge vertices, and the current vertices whose
    b(i) uses R1."""
    import json
    s = synth.build_symmetric(synth.config_small(nk=6, q_steps=1, nbnd=12, nocc=3, npw=60, nlf=7, no=31))
    ctx = rpa.Context(precision=rpa.PREC_MIXED)
    ctx.set_gvectors(s.miller, s.G, s.KC)
    ctx.set_symmetry(s.extra["nsym"], s.R, s.RI)
    ctx.load_basis(s.npw, s.igk, s.coeff, s.E)
    ctx.kmap(s.ktot, s.K1, s.R1, s.K2, s.R2, s.iG0)
    ctx.set_q(s.q, s.ilf, s.parG)
    So = orc.sloss_s0(orc.Bound(s))
    for swap in (1, 0):
        ctx.tune_import(json.dumps({"vertex": [{"mode": rpa.MODE_CHARGE, "nbnd": 12, "nocc": 3, "nlf32": 0,
                                                "ymax": 0, "swap": swap}]}))
        S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
        assert rel(S, So) < TOL, swap
    for pol in ("xx", "zy"):
        Sc, _ = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, pol))
        Sco, _ = orc.optabs_s0(orc.Bound(s, pol=pol))
        assert rel(Sc, Sco) < TOL, pol
    ctx.close()


@pytest.mark.parametrize("first,second,ymax", [("xx", "zz", 32), ("zz", "yy", 16)])
def test_prefetched_polarisation(synth, rpa, orc, first, second, ymax):
    """rpa_chi0_prefetch: the first chi0 computes the second polarisation's
    vertices in the same pass (three column blocks c | b1 c | b2 c); the second
    chi0 uses them.  Both S0 / Qeff against the oracle (Optabs.f90:291-471) at
    the mixed-path tolerance and against the same calls without the prefetch
    (equal up to FP32 rounding order); rpa_kk in between keeps the stash,
    rpa_set_q drops it."""
    import json
    s = synth.build(synth.config_small(nbnd=24, npw=150, nlf=40, lf="xyz", no=31))
    ctx = rpa.Context(precision=rpa.PREC_MIXED)
    ctx.load_system(s)
    ctx.tune_import(json.dumps({"vertex": [{"mode": rpa.MODE_CURRENT, "nbnd": 24, "nocc": 0, "nlf32": s.nlf // 32,
                                            "ymax": ymax, "swap": -1}]}))
    ref = {}
    for pol in (first, second):
        ref[pol] = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, pol))
    ctx.chi0_prefetch(second)
    S1, Q1 = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, first))
    ctx.kk(rpa.KK_OPTABS_COMPLEX, want=False)
    S2, Q2 = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, second))
    assert ctx.stage_times()["vertices"] < 0.05  # the stashed rows were used
    for pol, (S, Q) in ((first, (S1, Q1)), (second, (S2, Q2))):
        So, Qo = orc.optabs_s0(orc.Bound(s, pol=pol))
        assert rel(S, So) < TOL and rel(Q, Qo) < TOL, pol
        assert rel(S, ref[pol][0]) < 1e-6 and rel(Q, ref[pol][1]) < 1e-6, pol
    # a set_q between the two calls drops the stash: the second call recomputes
    ctx.chi0_prefetch(second)
    ctx.chi0(rpa.MODE_CURRENT, want=False, **rpa.optabs_args(s, first))
    ctx.set_q(s.q, s.ilf, s.parG)
    S3, _ = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, second))
    assert ctx.stage_times()["vertices"] > 0
    assert rel(S3, ref[second][0]) < 1e-6
    with pytest.raises(rpa.RpaError) as e:
        ctx.chi0_prefetch("yz")
    assert e.value.code == rpa.RPA_EINVAL
    ctx.close()


def test_prefetch_dropped_by_another_call(synth, rpa, orc):
    """The stash of a prefetched polarisation is dropped by any chi0 in
    between (a charge-mode call here): the later zz call computes its own
    vertices and still matches the oracle; a prefetch on an FP64 context is
    accepted and has no effect."""
    s = synth.build(synth.config_small(nbnd=16, npw=120, nlf=19, lf="xyz", no=21))
    ctx = rpa.Context(precision=rpa.PREC_MIXED)
    ctx.load_system(s)
    ctx.chi0_prefetch("zz")
    ctx.chi0(rpa.MODE_CURRENT, want=False, **rpa.optabs_args(s, "xx"))
    Sl, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    S, Q = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, "zz"))
    assert ctx.stage_times()["vertices"] > 0
    So, Qo = orc.optabs_s0(orc.Bound(s, pol="zz"))
    assert rel(S, So) < TOL and rel(Q, Qo) < TOL
    assert rel(Sl, orc.sloss_s0(orc.Bound(s))) < TOL
    ctx.close()
    f = rpa.Context(precision=rpa.PREC_FP64)
    f.load_system(s)
    f.chi0_prefetch("zz")
    S64, _ = f.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, "xx"))
    assert rel(S64, orc.optabs_s0(orc.Bound(s, pol="xx"))[0]) < 1e-11
    f.close()
