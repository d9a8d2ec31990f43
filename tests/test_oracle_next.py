"""Oracle restatements of the consumers after the hot path (CPU only): the
Optabs calc = 2 assembly (Pi, conductivity) and the KK transform of W with
its self-check, checked against closed forms."""
import numpy as np


def test_w1w2_single_spike(orc):
    no, d = 11, 0.1
    S = np.zeros((1, 1, no))
    S[0, 0, 4] = 1.0  # a spike at oj = 4 d
    W1, W2 = orc._w1w2(1, no, 0.0, d, S)
    assert np.isclose(W1[0, 0], -d / (4 * d)) and np.isclose(W2[0, 0], -W1[0, 0])
    for io in (2, 3, 7, no - 1):
        oi = (io - 1) * d
        W1, W2 = orc._w1w2(io, no, oi, d, S)
        assert np.isclose(W1[0, 0], d / (oi - 4 * d))
        assert np.isclose(W2[0, 0], d / (oi + 4 * d))
    # the row io never contributes to W1 at io (the else-if chain sets fact = 0)
    W1, _ = orc._w1w2(5, no, 4 * d, d, S)
    assert W1[0, 0] == 0.0


def test_kk_w_of_a_consistent_pair_is_small(orc):
    # W - V = a pole pair: Re and Im are a KK pair, so the self-check error is
    # a discretisation error only
    no, d, e0, g = 801, 0.01, 2.0, 0.2
    o = np.arange(no - 1) * d
    w = 1.0 / (o - e0 + 1j * g) - 1.0 / (o + e0 + 1j * g)
    V11 = 0.7
    WT = (w + V11).reshape(1, 1, -1)
    S0 = np.zeros((1, 1, no))
    S0[0, 0, -1] = -(1.0 / np.pi) * w[-1].imag
    Gp, Gm, chk = orc.kk_w(WT, S0, V11, d)
    assert chk[2] < 1.0  # percent
    assert np.isclose(chk[4], (WT[0, 0, 0] - V11).real / 2)
    np.testing.assert_allclose(Gp[0, 0].imag, WT[0, 0].imag)
    assert np.all(Gm.imag == 0)


def test_pi_assembly_matches_the_closed_form(orc):
    rng = np.random.default_rng(3)
    for nlf in (1, 4):
        nwo, d, eta, c0 = 30, 0.02, 0.05, 37.8
        chi0 = rng.standard_normal((nlf, nlf, nwo)) + 1j * rng.standard_normal((nlf, nlf, nwo))
        Q = rng.standard_normal((nlf, nlf)) + 1j * rng.standard_normal((nlf, nlf))
        pi11, sig, full = orc.pi_assembly(chi0, Q, d, eta, c0)
        oi = np.arange(nwo) * d
        intra = Q[..., None] * oi / (oi + 1j * eta)
        Pi = chi0 - chi0[..., :1].real + intra
        np.testing.assert_allclose(full, Pi, rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(pi11, Pi[0, 0], rtol=1e-13, atol=1e-13)
        inter = Pi[0, 0] if nlf > 1 else Pi[0, 0] - intra[0, 0]
        np.testing.assert_allclose(sig[0, 1:], c0 * inter.imag[1:] / oi[1:], rtol=1e-12)
        np.testing.assert_allclose(sig[1, 1:], c0 * intra[0, 0].imag[1:] / oi[1:], rtol=1e-12)
        assert sig[0, 0] == 0 and sig[1, 0] == 0


def _hex(synth, nk):
    a0, c0, V, KC = synth.hex_cell(2.46, 20.0)
    nsym, R, RI = synth.hex_symmetry()
    kI = synth.mp_ibz(KC, nk, R, nsym)
    miller, G = synth.g_list(KC, 3.5 ** 2)
    return KC, nsym, R, RI, kI, miller, G


def test_kmap_oracle_on_a_symmetric_grid(synth, orc):
    """genFBZ / findKinIBZ / findKQinBZ restatements on a hexagonal 9x9 grid
    with C6v: the FBZ covers the grid (points on the Wigner-Seitz boundary
    appear once per distinct image), every point and every K+Q is found."""
    KC, nsym, R, RI, kI, miller, G = _hex(synth, 9)
    ktot = orc.gen_fbz(kI, R, nsym, 1e-4)
    assert ktot.shape[0] >= 81 and np.allclose(ktot[:kI.shape[0]], kI)
    d = np.abs(ktot[:, None, :] - ktot[None, :, :]).max(axis=2)
    assert (d[np.triu_indices(ktot.shape[0], 1)] > 1e-4).all()
    R1, K1 = orc.find_k_ibz(ktot, kI, RI, nsym, 1e-4)
    assert (R1 > 0).all() and (K1 > 0).all()
    for ik in range(ktot.shape[0]):
        assert np.allclose(RI[R1[ik] - 1] @ ktot[ik], kI[K1[ik] - 1], atol=1e-4)
    q = KC.T[0] / 9
    iG0, R2, K2 = orc.find_kq(ktot, kI, RI, nsym, G, q, 1e-4)
    assert (iG0 > 0).all()
    for ik in range(ktot.shape[0]):
        # K+Q - G is an FBZ point whose image under RI_R2 is the IBZ point K2
        assert np.allclose(RI[R2[ik] - 1] @ (ktot[ik] + q - G[iG0[ik] - 1]), kI[K2[ik] - 1], atol=1e-4)


def test_kmap_oracle_reproduces_the_grid_bookkeeping(synth, orc):
    """Identity symmetry on the Gamma-centred grid of the synthetic systems:
    the restated search gives the K2 / iG0 that synth.q_kmap constructs."""
    s = synth.build(synth.config_small(nk=6, q_steps=1))
    for steps, steps2 in ((1, 0), (2, 1), (5, 3)):
        km = synth.q_kmap(s, steps, steps2)
        iG0, R2, K2 = orc.find_kq(s.ktot, s.ktot, s.RI, 1, s.G, km["q"], 1e-4)
        assert (K2 == km["K2"]).all() and (iG0 == km["iG0"]).all() and (R2 == 1).all()


def test_w_equals_v_times_inverse_epsilon(orc):
    """The identity behind the mixed path's Dyson step: for eps = I - chi0 V,
    eps^-1 chi0 V = eps^-1 - I, so the reference's W = V + V chi V (chi =
    eps^-1 chi0) equals V eps^-1.  Checked on the oracle's loop-for-loop gjel
    and genWT restatement with a random complex chi0 and a real symmetric V."""
    rng = np.random.default_rng(7)
    n, nw = 9, 5
    A = rng.standard_normal((n, n))
    Vm = A @ A.T + n * np.eye(n)  # real symmetric, well conditioned
    chi = rng.standard_normal((n, n, nw)) + 1j * rng.standard_normal((n, n, nw))
    chi *= 0.5
    WT, Ei, rc = orc.dyson(chi, np.ascontiguousarray(Vm.T), fast_wt=False)
    assert rc == 0
    for w in range(nw):
        W = orc.fortran_mat(WT[:, :, w])
        E = orc.fortran_mat(Ei[:, :, w])
        C = orc.fortran_mat(chi[:, :, w])
        eps = np.eye(n) - C @ Vm
        assert np.allclose(E @ eps, np.eye(n), atol=1e-10)
        VE = Vm @ E
        assert np.max(np.abs(W - VE)) <= 1e-10 * np.max(np.abs(W))


def test_dyson_conditioning_on_decayed_basis(synth, orc, rpa):
    """On a basis whose coefficients fall by 8 decades to the cutoff, the
    Dyson step (eps = 1 - chi0 V, gjel, W = V + V chi V; Sloss.f90:452-481)
    amplifies a relative error of chi0 several hundred times: scaling the
    oracle's chi0 by 1 + 1e-6 moves W by more than 1e-4 (normwise) and Im
    eps^-1_00 by more than 1e-4 at some frequency above 1e-3 of its maximum,
    while on the flat basis the same change moves both by a few 1e-6.  This is
    the FP64 oracle alone (no GPU), so it is a property of the problem: any
    chi0 carrying ~1e-6 relative error gives W errors of this size there."""
    out = {}
    for dec in (0.0, 8.0):
        s = synth.build(synth.config_grid24(env_decades=dec))
        chio = orc.kk_sloss(orc.sloss_s0(orc.Bound(s)), s.domega)
        V = orc.genV(s)
        W0, E0, rc0 = orc.dyson(chio, V, fast_wt=True)
        W1, E1, rc1 = orc.dyson(np.ascontiguousarray(chio * (1.0 + 1e-6)), V, fast_wt=True)
        assert rc0 == 0 and rc1 == 0
        out[dec] = (rpa.errstats(W1, W0)["normwise"],
                    rpa.errstats(E1[0, 0].imag, E0[0, 0].imag, floor=1e-3)["elem_max"])
    assert out[0.0][0] < 1e-5 and out[0.0][1] < 1e-5
    assert out[8.0][0] > 1e-4 and out[8.0][1] > 1e-4
