"""GPU: batched W requests (rpa_batch) -- per-request setup, then one CUDA
graph with a grouped-tile S0 launch per tile shape and the KK / Dyson stages
of every request -- against the same requests run one by one on a mixed
context (identical kernels, so equal to rounding) and, for the request with
the system's own q and local fields, against the oracle (Sloss.f90:292-481:
S0, KK, gjel, W) at the mixed-path tolerance (1e-5: W normwise, Im eps^-1_00
element-wise above 1e-3 of its maximum)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _requests(synth, rpa, s):
    reqs = []
    # (q grid steps, NGloc, nw): NGloc 131 / 40 / 19 / 100 fall on different tile shapes
    for steps, nlf, no in ((1, 131, 41), (2, 40, 41), (3, 19, 31), (1, 100, 31)):
        km = synth.q_kmap(s, steps)
        if steps == 1 and nlf == s.nlf:
            ilf, par = s.ilf, s.parG
        else:
            ilf, par = synth.local_fields(s, km["q"], 1e9, lf="xyz", nmax=nlf)
        domega = s.domega * (s.no - 1) / (no - 1)
        args = dict(no=no, domega=domega, eta=s.eta, Vcell=s.Vcell, Gcar=s.Gcar, nocc=s.nocc)
        reqs.append(dict(kmap=km, ilf=ilf, parG=par, args=args, c0=s.c0, eps=s.cfg.eps))
    return reqs


def _one_by_one(rpa, ctx, r):
    km = r["kmap"]
    ctx.kmap(km["ktot"], km["K1"], km["R1"], km["K2"], km["R2"], km["iG0"])
    ctx.set_q(km["q"], r["ilf"], r["parG"])
    ctx.chi0(rpa.MODE_CHARGE, want=False, **r["args"])
    ctx.kk(rpa.KK_SLOSS_REAL, want=False)
    WT, _, head = ctx.dyson(r["c0"], r["eps"], want_wt=True)
    return WT, head


def test_batch_matches_single_requests_and_oracle(synth, rpa, orc):
    s = synth.build(synth.config_small(npw=200, nlf=131, lf="xyz", no=41))
    parent = rpa.Context(precision=rpa.PREC_MIXED)
    parent.load_system(s)
    reqs = _requests(synth, rpa, s)
    batch = rpa.Batch(parent, max_q=4)
    for run in range(2):  # twice: the second run reuses the contexts and the item table
        res = batch.run(reqs, want_wt=True)
        info = batch.info()
        assert info["groups"] >= 2 and info["graph_nodes"] > len(reqs)
        single = rpa.shared_context(parent)
        for i, (r, (st, out)) in enumerate(zip(reqs, res)):
            assert st == rpa.RPA_OK, (i, batch.last_error())
            WT1, head1 = _one_by_one(rpa, single, r)
            assert np.max(np.abs(out["WT"] - WT1)) <= 1e-12 * np.max(np.abs(WT1)), (run, i)
            assert np.max(np.abs(out["head"] - head1)) <= 1e-12 * np.max(np.abs(head1)), (run, i)
        single.close()
    # request 0 is the system's own q-point and local fields: against the oracle
    So = orc.sloss_s0(orc.Bound(s))
    WTo, Eio, rc = orc.dyson(orc.kk_sloss(So, s.domega), orc.genV(s), fast_wt=True)
    assert rc == 0
    out = res[0][1]
    assert rpa.errstats(out["WT"], WTo)["normwise"] < TOL
    e = rpa.errstats(out["head"].imag, Eio[0, 0, :].imag, floor=1e-3)
    assert e["elem_max"] < TOL, e
    batch.close()
    parent.close()


def test_two_batches_alternating(synth, rpa):
    """launch / wait halves: two batches on one parent, the second launched
    while the first's graph may still run, give the results of run()."""
    s = synth.build(synth.config_small(npw=200, nlf=131, lf="xyz", no=41))
    parent = rpa.Context(precision=rpa.PREC_MIXED)
    parent.load_system(s)
    reqs = _requests(synth, rpa, s)
    ref = rpa.Batch(parent, max_q=4)
    want = [o["head"] for _, o in ref.run(reqs)]
    ref.close()
    a, b = rpa.Batch(parent, max_q=2), rpa.Batch(parent, max_q=2)
    a.launch(reqs[:2])
    b.launch(reqs[2:])
    got = [o["head"] for _, o in a.wait()] + [o["head"] for _, o in b.wait()]
    for g, w in zip(got, want):
        assert np.max(np.abs(g - w)) <= 1e-12 * np.max(np.abs(w))
    with pytest.raises(rpa.RpaError) as e:
        a.wait()  # nothing pending
    a.close()
    b.close()
    parent.close()


def test_batch_rejects_other_requests(synth, rpa):
    s = synth.build(synth.config_small())
    parent = rpa.Context(precision=rpa.PREC_MIXED)
    parent.load_system(s)
    batch = rpa.Batch(parent, max_q=2)
    r = _requests(synth, rpa, synth.build(synth.config_small(npw=200, nlf=131, lf="xyz", no=41)))[:3]
    with pytest.raises(rpa.RpaError) as e:
        batch.run(r)  # three requests for two slots
    assert e.value.code == rpa.RPA_EINVAL
    batch.close()
    fp = rpa.Context()
    fp.load_system(s)
    with pytest.raises(rpa.RpaError) as e:
        rpa.Batch(fp, max_q=1)
    assert e.value.code == rpa.RPA_ESTATE
    fp.close()
    parent.close()
