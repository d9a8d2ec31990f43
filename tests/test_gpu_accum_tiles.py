"""GPU: the tile variants of the mixed path's S0 accumulation and their
autotuner.

Every (G-tile rows, frequency rows per CTA) variant of the warp-specialised
kernel computes the same S0 (Sloss.f90:407-418, Optabs.f90:387-421) in a
different tiling; each is forced in turn (opts.reserved[2]) and checked
against the oracle at the mixed-path tolerance, on NGloc that fits one tile
of some variants and spans several tiles of others (the symmetric tile-pair
skip included).  rpa_autotune keeps the fastest variant per (S0 kind, NGloc,
nw / 64) and its table survives an export / import round trip.

Tolerance: 1e-5 normwise max relative error (max |a - b| / max |b|)."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module", params=[40, 131])
def system(request, synth, orc):
    s = synth.build(synth.config_small(npw=200, nlf=request.param, lf="xyz", no=21))
    refs = {"charge": orc.sloss_s0(orc.Bound(s)), "xx": orc.optabs_s0(orc.Bound(s, pol="xx"))}
    return s, refs


@pytest.mark.parametrize("variant", [v for v in [(96, 2), (128, 1), (64, 2), (48, 2), (32, 2)]])
def test_real_s0_every_tile_variant(system, rpa, variant):
    assert variant in rpa.ACC_VARIANTS["real"]
    s, refs = system
    ctx = rpa.Context(precision=rpa.PREC_MIXED, acc_tile=variant)
    ctx.load_system(s)
    S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    assert ctx.accum_tile()[0] == variant[0]
    assert rel(S, refs["charge"]) < TOL, variant
    ctx.close()


@pytest.mark.parametrize("variant", [(96, 1), (64, 1), (32, 2)])
def test_complex_s0_every_tile_variant(system, rpa, variant):
    assert variant in rpa.ACC_VARIANTS["complex"]
    s, refs = system
    ctx = rpa.Context(precision=rpa.PREC_MIXED, acc_tile=variant)
    ctx.load_system(s)
    S, Q = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, "xx"))
    assert ctx.accum_tile() == variant
    So, Qo = refs["xx"]
    assert rel(S, So) < TOL, variant
    assert rel(Q, Qo) < TOL, variant
    ctx.close()


def test_forced_tile_rules(synth, rpa, orc):
    """A variant of the other S0 kind is refused (RPA_EINVAL); the yz pair
    (M2 != M) keeps the default 96-row tiles whatever is forced."""
    s = synth.build(synth.config_small(npw=200, nlf=40, lf="xyz", no=21))
    ctx = rpa.Context(precision=rpa.PREC_MIXED, acc_tile=(128, 1))
    ctx.load_system(s)
    with pytest.raises(rpa.RpaError) as e:
        ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, "xx"))
    assert e.value.code == rpa.RPA_EINVAL
    ctx.close()
    ctx = rpa.Context(precision=rpa.PREC_MIXED, acc_tile=(32, 2))
    ctx.load_system(s)
    S, Q = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, "yz"))
    assert ctx.accum_tile() == (96, 1)
    So, Qo = orc.optabs_s0(orc.Bound(s, pol="yz"))
    assert rel(S, So) < TOL and rel(Q, Qo) < TOL
    ctx.close()


def test_autotune_accumulation_table(synth, rpa, orc):
    s = synth.build(synth.config_small(npw=200, nlf=40, lf="xyz", no=21))
    ctx = rpa.Context(precision=rpa.PREC_MIXED)
    ctx.load_system(s)
    ctx.autotune(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    ctx.autotune(rpa.MODE_CURRENT, **rpa.optabs_args(s, "xx"))
    acc = json.loads(ctx.tune_export())["accum"]
    keys = {(e["cplx"], e["nlf"], e["nw64"]) for e in acc}
    assert keys == {(0, 40, s.no // 64), (1, 40, (2 * s.no + 1) // 64)}
    for e in acc:
        kind = "complex" if e["cplx"] else "real"
        assert (e["gb"], e["nio"]) in [tuple(v) for v in rpa.ACC_VARIANTS[kind]] and e["ms"] > 0
    # the tuned choice is what later calls use, and it gives the right S0
    S, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    real = [e for e in acc if e["cplx"] == 0][0]
    assert ctx.accum_tile()[0] == real["gb"]
    assert rel(S, orc.sloss_s0(orc.Bound(s))) < TOL
    text = ctx.tune_export()
    other = rpa.Context(precision=rpa.PREC_MIXED)
    other.tune_import(text)
    assert json.loads(other.tune_export())["accum"] == acc
    with pytest.raises(rpa.RpaError):
        other.tune_import('{"vertex": [], "accum": [{"cplx": 0, "nlf": 40, "nw64": 0, "gb": 80, "nio": 2}]}')
    for c in (ctx, other):
        c.close()


def test_row_order_and_its_limit(synth, rpa, orc):
    """The frequency-row blocks of an accumulation launch run costliest window
    first (k_row_order sorts up to 4096 blocks); a launch with more blocks
    keeps index order.  no = 2100: the complex S0 on forced one-row (96, 1)
    tiles has 4201 blocks (index order); with the default tile and for the
    real S0 the blocks are sorted.  All against the oracle at the mixed-path
    tolerance."""
    s = synth.build(synth.config_small(npw=200, nlf=19, no=2100))
    So, Qo = orc.optabs_s0(orc.Bound(s, pol="xx"))
    Ro = orc.sloss_s0(orc.Bound(s))
    ctx = rpa.Context(precision=rpa.PREC_MIXED, acc_tile=(96, 1))
    ctx.load_system(s)
    S, Q = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, "xx"))
    assert ctx.accum_tile() == (96, 1)
    assert S.shape == So.shape and rel(S, So) < TOL and rel(Q, Qo) < TOL
    ctx.close()
    ctx = rpa.Context(precision=rpa.PREC_MIXED)
    ctx.load_system(s)
    S, Q = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, "xx"))
    assert rel(S, So) < TOL and rel(Q, Qo) < TOL
    R, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
    assert rel(R, Ro) < TOL
    ctx.close()
