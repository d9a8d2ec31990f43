"""GPU parity of the consumers after the hot path, FP64 path against the
oracle: the Optabs calc = 2 assembly (Pi_11 spectrum, conductivities, full
Pi; to 1e-11 like chi0) and the KK transform of W with its self-check (to
1e-9 like W)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-11
TOL_W = 1e-9


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("nlf", [7, 1])
def test_pi_assembly(synth, rpa, orc, nlf):
    s = synth.build(synth.config_small(nlf=nlf))
    ctx = rpa.Context()
    ctx.load_system(s)
    ctx.chi0(rpa.MODE_CURRENT, want=False, **rpa.optabs_args(s, "xx"))
    ctx.kk(rpa.KK_OPTABS_COMPLEX, want=False)
    eta_intra, c0 = 0.01 / 27.211386, s.c0
    p11, sig, full = ctx.pi(eta_intra, c0, want_full=True)
    So, Qo = orc.optabs_s0(orc.Bound(s, pol="xx"))
    p11o, sigo, fullo = orc.pi_assembly(orc.kk_optabs(So, s.domega), Qo, s.domega, eta_intra, c0)
    assert rel(p11, p11o) < TOL
    assert rel(full, fullo) < TOL
    assert rel(sig[0], sigo[0]) < TOL and rel(sig[1], sigo[1]) < TOL
    ctx.close()


def test_kk_of_w_and_self_check(synth, rpa, orc):
    s = synth.build(synth.config_small())
    ctx = rpa.Context()
    ctx.load_system(s)
    ctx.chi0(rpa.MODE_CHARGE, want=False, **rpa.sloss_args(s))
    ctx.kk(rpa.KK_SLOSS_REAL, want=False)
    ctx.dyson(s.c0, s.cfg.eps, want_wt=False, want_head=False)
    gp, gm, chk = ctx.kk_w()
    So = orc.sloss_s0(orc.Bound(s))
    V = orc.genV(s)
    WTo, _, rc = orc.dyson(orc.kk_sloss(So, s.domega), V, fast_wt=True)
    assert rc == 0
    gpo, gmo, chko = orc.kk_w(WTo, So, float(V[0, 0]), s.domega)
    assert rel(gp, gpo) < TOL_W and rel(gm, gmo) < TOL_W
    assert abs(chk[1] - chko[1]) <= TOL_W * abs(chko[1])
    assert abs(chk[0] - chko[0]) <= 1e-8 * abs(chko[1])
    assert abs(chk[3] - chko[3]) <= TOL_W * max(abs(chko[3]), 1e-300)
    assert abs(chk[4] - chko[4]) <= TOL_W * max(abs(chko[4]), 1e-300)
    ctx.close()
