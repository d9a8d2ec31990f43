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


def _hex(synth, nk):
    a0, c0, V, KC = synth.hex_cell(2.46, 20.0)
    nsym, R, RI = synth.hex_symmetry()
    kI = synth.mp_ibz(KC, nk, R, nsym)
    miller, G = synth.g_list(KC, 3.5 ** 2)
    return KC, nsym, R, RI, kI, miller, G


@pytest.mark.parametrize("nk", [6, 12])
def test_kmap_on_the_device_equals_the_restated_search(synth, rpa, orc, nk):
    """rpa_gen_fbz / rpa_find_k_ibz / rpa_find_kq against the oracle's
    loop-for-loop genFBZ / findKinIBZ / findKQinBZ: identical points and
    indices (C6v, hexagonal grid, q along Gamma-M, Gamma-K and off-axis)."""
    KC, nsym, R, RI, kI, miller, G = _hex(synth, nk)
    ctx = rpa.Context()
    ctx.set_gvectors(miller, G, KC)
    ctx.set_symmetry(nsym, R, RI)
    ktot = ctx.gen_fbz(kI, 1e-4)
    kto = orc.gen_fbz(kI, R, nsym, 1e-4)
    assert ktot.shape == kto.shape and (ktot == kto).all()
    R1, K1 = ctx.find_k_ibz(ktot, kI, 1e-4)
    R1o, K1o = orc.find_k_ibz(kto, kI, RI, nsym, 1e-4)
    assert (R1 == R1o).all() and (K1 == K1o).all()
    b = KC.T
    for q in (b[0] / nk, (b[0] + b[1]) / nk, (2 * b[0] + b[1]) / nk):
        got = ctx.find_kq(ktot, kI, q, 1e-4)
        ref = orc.find_kq(kto, kI, RI, nsym, G, q, 1e-4)
        for a, r in zip(got, ref):
            assert (a == r).all()
    ctx.close()


def test_kmap_on_the_device_reproduces_the_grid_bookkeeping(synth, rpa):
    s = synth.build(synth.config_small(nk=6, q_steps=1))
    ctx = rpa.Context()
    ctx.set_gvectors(s.miller, s.G, s.KC)
    assert (ctx.gen_fbz(s.ktot) == s.ktot).all()
    for steps, steps2 in ((1, 0), (2, 1), (5, 3)):
        km = synth.q_kmap(s, steps, steps2)
        iG0, R2, K2 = ctx.find_kq(s.ktot, s.ktot, km["q"])
        assert (K2 == km["K2"]).all() and (iG0 == km["iG0"]).all() and (R2 == 1).all()
    ctx.close()


def test_kmap_off_grid_q_is_not_found(synth, rpa):
    """A q that is not a grid vector: the reference stops ('Can not find wave
    vector K+Q'); the device search returns RPA_ENOTFOUND."""
    KC, nsym, R, RI, kI, miller, G = _hex(synth, 6)
    ctx = rpa.Context()
    ctx.set_gvectors(miller, G, KC)
    ctx.set_symmetry(nsym, R, RI)
    ktot = ctx.gen_fbz(kI)
    with pytest.raises(rpa.RpaError) as e:
        ctx.find_kq(ktot, kI, 0.37 * KC.T[0] / 6)
    assert e.value.code == rpa.RPA_ENOTFOUND
    ctx.close()


def test_corrfun_and_wt_files_from_the_device_path(synth, rpa, tmp_path):
    """Optabs calc = 1 output written from the device S0 / Qeff and read back as
    calc = 2 would (values rounded to the files' 10 decimals), and the Sloss
    W_Qi file of the device WT."""
    s = synth.build(synth.config_small())
    ctx = rpa.Context()
    ctx.load_system(s)
    S, Q = ctx.chi0(rpa.MODE_CURRENT, **rpa.optabs_args(s, "xx"))
    p0, p1 = str(tmp_path / "Corrfun_xx"), str(tmp_path / "Qeff_xx")
    rpa.write_corrfun(p0, p1, S, Q, s.domega)
    Sr, Qr = rpa.read_corrfun(p0, p1, s.no, s.nlf)
    for a, b in ((Sr, S), (Qr, Q)):
        assert np.abs(a.real - b.real).max() <= 5.0001e-11 and np.abs(a.imag - b.imag).max() <= 5.0001e-11
    ctx.chi0(rpa.MODE_CHARGE, want=False, **rpa.sloss_args(s))
    ctx.kk(rpa.KK_SLOSS_REAL, want=False)
    WT, _, _ = ctx.dyson(s.c0, s.cfg.eps)
    rpa.write_wt(str(tmp_path / "W_Q1"), WT, s.domega)
    vals = " ".join(open(tmp_path / "W_Q1").read().splitlines()[1:]).split()
    got = np.array([float(v) for v in vals]).reshape(-1, 2)
    ref = np.array([[WT[j, i, 0].real, WT[j, i, 0].imag] for i in range(s.nlf) for j in range(s.nlf)])
    assert np.abs(got - ref).max() <= 5.0001e-6
    ctx.close()
