"""Serving on one resident basis: contexts that share the basis, and the
request loop with continuous batching (rpa_server_*).

A request's result must not depend on what else runs: the same requests are
served one at a time (one slot) and all at once (three slots, submitted
together so that they overlap on the GPU), and the outputs must agree to
1e-12 relative (the kernels are deterministic, so they are expected to be
identical).  One W request of an FP64 server is also checked against the CPU
oracle's Sloss chain (W to 1e-9, as the FP64 parity tests)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_SAME = 1e-12
TOL_DYSON = 1e-9


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _requests(rpa, synth, s):
    """W (Sloss) and chi0 (Optabs xx / zz) requests of different q, local-field
    cutoffs and frequency grids."""
    out = []
    # cutoffs (2pi/a0)^2 giving 9-26 local fields on the 6x6 system
    for i, (steps, g2, no, kind) in enumerate([(1, 1.0, 41, "W"), (2, 1.0, 31, "chi0"), (3, 0.5, 61, "W"),
                                               (1, 0.5, 21, "chi0"), (4, 1.0, 41, "W"), (2, 0.5, 51, "chi0")]):
        km = synth.q_kmap(s, steps)
        ilf, par = synth.local_fields(s, km["q"], g2, lf="xyz", nmax=24)
        domega = s.domega * (s.no - 1) / (no - 1)
        if kind == "W":
            args = dict(no=no, domega=domega, eta=s.eta, Vcell=s.Vcell, Gcar=s.Gcar, nocc=s.nocc)
            out.append(dict(kind=rpa.REQ_W, kmap=km, ilf=ilf, parG=par, args=args, mode=rpa.MODE_CHARGE,
                            kk_variant=rpa.KK_SLOSS_REAL, c0=s.c0, eps=s.cfg.eps, want_wt=True))
        else:
            a = rpa.optabs_args(s, "xx" if i % 2 else "zz")
            a.update(no=no, domega=domega)
            out.append(dict(kind=rpa.REQ_CHI0, kmap=km, ilf=ilf, parG=par, args=a, mode=rpa.MODE_CURRENT,
                            kk_variant=rpa.KK_OPTABS_COMPLEX, want_s0=True))
    return out


@pytest.fixture(scope="module")
def parent(synth, rpa):
    s = synth.build(synth.config_small())
    ctx = rpa.Context(precision=rpa.PREC_MIXED)
    ctx.load_system(s)
    yield s, ctx
    ctx.close()


def test_results_same_alone_and_in_the_mix(parent, rpa, synth):
    s, ctx = parent
    reqs = _requests(rpa, synth, s)
    assert len({r["ilf"].size for r in reqs}) > 1 and len({r["args"]["no"] for r in reqs}) > 1
    alone = []
    srv = rpa.Server(ctx, nslots=1, mem_bytes=1e9)
    for r in reqs:
        alone.append(srv.wait(srv.submit(**r))[0])
    srv.close()
    srv = rpa.Server(ctx, nslots=3, mem_bytes=1e9)
    ids = [srv.submit(**r) for r in reqs]
    mixed = [srv.wait(i) for i in ids]
    srv.close()
    for (outs, times), ref in zip(mixed, alone):
        assert times[0] >= times[2] >= 0.0 and times[1] >= 0.0
        assert set(outs) == set(ref)
        for k in ref:
            assert np.abs(ref[k]).max() > 0, k
            assert rel(outs[k], ref[k]) <= TOL_SAME, k


def test_batching_worker_results_same_as_alone(parent, rpa, synth):
    """rpa_server_create_batched: the W requests (without chi0 output) that the
    batching worker runs as one rpa_batch give the W and eps^-1_11 of the
    same requests served one at a time, and the chi0 requests are still
    served by the slot workers."""
    s, ctx = parent
    reqs = _requests(rpa, synth, s)
    for r in reqs:
        if r["kind"] == rpa.REQ_W:
            r["want_chi0"] = False
    alone = []
    srv = rpa.Server(ctx, nslots=1, mem_bytes=1e9)
    for r in reqs:
        alone.append(srv.wait(srv.submit(**r))[0])
    srv.close()
    # one slot worker that is kept busy by a first chi0 request, so the W
    # requests queued behind it go to the batching worker
    srv = rpa.Server(ctx, nslots=1, mem_bytes=1e9, batch_q=4)
    ids = [srv.submit(**r) for r in reqs]
    mixed = [srv.wait(i)[0] for i in ids]
    n_batched = srv.batched_count()
    srv.close()
    assert n_batched >= 1
    for outs, ref in zip(mixed, alone):
        assert set(outs) == set(ref)
        for k in ref:
            assert rel(outs[k], ref[k]) <= TOL_SAME, k


def test_server_request_equals_a_context_call(parent, rpa, synth):
    s, ctx = parent
    r = _requests(rpa, synth, s)[2]  # W request, q = 3 grid steps
    srv = rpa.Server(ctx, nslots=2, mem_bytes=1e9)
    outs, _ = srv.wait(srv.submit(**r))
    srv.close()
    c = rpa.shared_context(ctx)
    km = r["kmap"]
    c.kmap(km["ktot"], km["K1"], km["R1"], km["K2"], km["R2"], km["iG0"])
    c.set_q(km["q"], r["ilf"], r["parG"])
    c.chi0(rpa.MODE_CHARGE, want=False, **r["args"])
    chi = c.kk(rpa.KK_SLOSS_REAL)
    WT, _, head = c.dyson(r["c0"], r["eps"])
    c.close()
    assert rel(outs["chi0"], chi) <= TOL_SAME
    assert rel(outs["WT"], WT) <= TOL_SAME
    assert rel(outs["head"], head) <= TOL_SAME


def test_fp64_server_matches_the_oracle(synth, rpa, orc):
    s = synth.build(synth.config_small(q_steps=2))
    ctx = rpa.Context(precision=rpa.PREC_FP64)
    ctx.load_system(s)
    srv = rpa.Server(ctx, nslots=2, mem_bytes=1e9)
    km = synth.q_kmap(s, 2)
    args = dict(no=s.no, domega=s.domega, eta=s.eta, Vcell=s.Vcell, Gcar=s.Gcar, nocc=s.nocc)
    rid = srv.submit(kind=rpa.REQ_W, kmap=km, ilf=s.ilf, parG=s.parG, args=args, mode=rpa.MODE_CHARGE,
                     kk_variant=rpa.KK_SLOSS_REAL, c0=s.c0, eps=s.cfg.eps, want_wt=True)
    outs, _ = srv.wait(rid)
    srv.close()
    b = orc.Bound(s)
    chio = orc.kk_sloss(orc.sloss_s0(b), s.domega)
    WTo, Eio, rc = orc.dyson(chio, orc.genV(s), fast_wt=True)
    assert rc == 0
    assert rel(outs["WT"], WTo) < TOL_DYSON
    assert rel(outs["head"], Eio[0, 0, :]) < TOL_DYSON
    ctx.close()


def test_shared_basis_is_protected(parent, rpa):
    s, ctx = parent
    c = rpa.shared_context(ctx)
    with pytest.raises(rpa.RpaError) as e:
        c.load_basis(s.npw, s.igk, s.coeff, s.E)
    assert e.value.code == rpa.RPA_ESTATE
    with pytest.raises(rpa.RpaError) as e:
        ctx.load_basis(s.npw, s.igk, s.coeff, s.E)
    assert e.value.code == rpa.RPA_ESTATE
    assert ctx.L.rpa_destroy(ctx.h) == rpa.RPA_ESTATE
    c.close()


def test_a_failing_request_does_not_stop_the_server(parent, rpa, synth):
    """A request whose chi0 arguments are invalid fails with its own error code;
    the requests around it are served normally and unchanged."""
    s, ctx = parent
    reqs = _requests(rpa, synth, s)[:3]
    srv = rpa.Server(ctx, nslots=2, mem_bytes=1e9)
    ref = [srv.wait(srv.submit(**r))[0] for r in reqs]
    bad = dict(reqs[0])
    bad["args"] = dict(bad["args"], nocc=0)  # Sloss needs 1 <= nocc < nbnd
    ids = [srv.submit(**reqs[0]), srv.submit(**bad), srv.submit(**reqs[1]), srv.submit(**reqs[2])]
    out0 = srv.wait(ids[0])[0]
    with pytest.raises(rpa.RpaError) as e:
        srv.wait(ids[1])
    assert e.value.code == rpa.RPA_EINVAL
    outs = [out0, srv.wait(ids[2])[0], srv.wait(ids[3])[0]]
    srv.close()
    for o, r in zip(outs, ref):
        for k in r:
            assert rel(o[k], r[k]) <= TOL_SAME, k
