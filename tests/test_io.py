"""The on-disk formats either side of the path (host code, no GPU): the QE 6
binary reader (loadG / loadCs_full of Modules/io_qe.f90) against files written
here record by record, and the Optabs Corrfun / Sloss W_Qi text formats
against a restatement of Fortran F editing."""
import os
import struct

import numpy as np
import pytest


def _rec(f, payload: bytes):
    f.write(struct.pack("<i", len(payload)))
    f.write(payload)
    f.write(struct.pack("<i", len(payload)))


def _write_charge_density(path, mill, b):
    with open(path, "wb") as f:
        _rec(f, struct.pack("<iii", 0, mill.shape[0], 1))          # gamma_only, ngm, nspin
        _rec(f, np.asarray(b, dtype="<f8").tobytes())               # b1, b2, b3
        _rec(f, np.ascontiguousarray(mill, dtype="<i4").tobytes())  # mill(3, ngm)
        _rec(f, np.zeros(2 * mill.shape[0]).tobytes())              # rho (not read)


def _write_wfc(path, ik, xk, mill, evc, npol=1, igwx=None):
    igwx = mill.shape[0] if igwx is None else igwx
    with open(path, "wb") as f:
        _rec(f, struct.pack("<i3diid", ik, *xk, 1, 0, 1.0))         # ik, xk, ispin, gamma_only, scalef
        _rec(f, struct.pack("<iiii", igwx + 7, igwx, npol, evc.shape[0]))
        _rec(f, np.eye(3).tobytes())
        _rec(f, np.ascontiguousarray(mill, dtype="<i4").tobytes())
        for band in evc:
            _rec(f, np.ascontiguousarray(band, dtype="<c16").tobytes())


@pytest.fixture
def save_dir(tmp_path, synth):
    a0, c0, V, KC = synth.hex_cell(2.46, 20.0)
    mill, G = synth.g_list(KC, 2.0 ** 2)
    _write_charge_density(tmp_path / "charge-density.dat", mill, KC.T)
    rng = np.random.default_rng(3)
    wfcs = []
    for ik, npw in ((1, 37), (2, 41)):
        m = mill[rng.permutation(mill.shape[0])[:npw]]
        evc = rng.standard_normal((5, npw)) + 1j * rng.standard_normal((5, npw))
        xk = rng.standard_normal(3)
        _write_wfc(tmp_path / f"wfc{ik}.dat", ik, xk, m, evc)
        wfcs.append((m, evc, xk))
    return str(tmp_path), KC, mill, wfcs


def test_qe_gvectors(save_dir, rpa):
    d, KC, mill, _ = save_dir
    m, G, par = rpa.qe_read_gvectors(d, KC)
    assert (m == mill).all()
    ref = np.zeros_like(G)
    for g in range(mill.shape[0]):  # G(n,iG) = sum_m KC(n,m) Gi(m,iG) from zero, m in order
        for n in range(3):
            s = 0.0
            for k in range(3):
                s = s + float(KC[n, k]) * float(mill[g, k])
            ref[g, n] = s
    assert (G == ref).all()
    assert (par == mill[:, 2]).all()


def test_qe_wavefunctions(save_dir, rpa):
    d, KC, mill, wfcs = save_dir
    for ik, (m, evc, xk) in enumerate(wfcs, start=1):
        c, mm, x = rpa.qe_read_wfc(d, ik, npwx=48, nbnd=4)
        assert (c[:, :m.shape[0]] == evc[:4]).all() and (c[:, m.shape[0]:] == 0).all()
        assert (mm == m).all() and (x == xk).all()


def test_qe_reader_errors(save_dir, rpa, tmp_path):
    d, KC, mill, wfcs = save_dir
    with pytest.raises(rpa.RpaError):
        rpa.qe_read_wfc(d, 3)                       # no such file
    with pytest.raises(rpa.RpaError) as e:
        rpa.qe_read_wfc(d, 1, npwx=48, nbnd=9)      # more bands than the file holds
    assert "only 5 bands" in str(e.value)
    with pytest.raises(rpa.RpaError):
        rpa.qe_read_wfc(d, 1, npwx=20)              # igwx above npwx
    m, evc, xk = wfcs[0]
    _write_wfc(os.path.join(d, "wfc4.dat"), 4, xk, m, evc, npol=2)
    with pytest.raises(rpa.RpaError):
        rpa.qe_read_wfc(d, 4)                       # spinor file
    raw = open(os.path.join(d, "wfc2.dat"), "rb").read()
    open(os.path.join(d, "wfc5.dat"), "wb").write(raw[:-20])
    with pytest.raises(rpa.RpaError):
        rpa.qe_read_wfc(d, 5)                       # truncated last record
    with pytest.raises(rpa.RpaError):
        rpa.qe_read_gvectors(str(tmp_path / "nowhere"), KC)


def fortran_f(x: float, w: int, d: int) -> str:
    """Fortran Fw.d output editing: right-aligned, d decimals, asterisks when the
    value does not fit the field."""
    s = f"{x:{w}.{d}f}"
    return "*" * w if len(s) > w else s


def test_corrfun_round_trip_and_layout(rpa, tmp_path):
    rng = np.random.default_rng(9)
    no, nlf = 4, 3
    S0 = (rng.standard_normal((nlf, nlf, 2 * no + 1)) + 1j * rng.standard_normal((nlf, nlf, 2 * no + 1))) * 1e-3
    S0[0, 1, 2] = -1.25e-12 + 3.5e5j      # a value that rounds to -0 and one that overflows F15.10
    Q = rng.standard_normal((nlf, nlf)) + 1j * rng.standard_normal((nlf, nlf))
    p0, p1 = str(tmp_path / "Corrfun_xx"), str(tmp_path / "Qeff_xx")
    rpa.write_corrfun(p0, p1, S0, Q, domega=0.01)
    lines = open(p0).read().splitlines()
    assert len(lines) == (2 * no + 1) * (nlf * nlf + 1)
    # memory of S0 is Fortran S0(io, iG, jG): S0[jG, iG, io]
    k = 0
    for io in range(2 * no + 1):
        assert lines[k].split()[0] == "omega=" and float(lines[k].split()[1]) == pytest.approx((io - no) * 0.01)
        k += 1
        for iG in range(nlf):
            for jG in range(nlf):
                v = S0[jG, iG, io]
                assert lines[k] == fortran_f(v.real, 15, 10) + fortran_f(v.imag, 15, 10)
                k += 1
    ql = open(p1).read().splitlines()
    assert ql == [fortran_f(Q[j, i].real, 15, 10) + fortran_f(Q[j, i].imag, 15, 10)
                  for i in range(nlf) for j in range(nlf)]
    with pytest.raises(rpa.RpaError):      # the overflow field cannot be read back, as in Fortran
        rpa.read_corrfun(p0, p1, no, nlf)
    S0[0, 1, 2] = 0.0
    rpa.write_corrfun(p0, p1, S0, Q, domega=0.01)
    S, Qr = rpa.read_corrfun(p0, p1, no, nlf)
    for a, b in ((S, S0), (Qr, Q)):  # each part rounded to 10 decimals
        assert np.abs(a.real - b.real).max() <= 5.0001e-11 and np.abs(a.imag - b.imag).max() <= 5.0001e-11


def test_wt_file_layout(rpa, tmp_path):
    rng = np.random.default_rng(2)
    nlf, nw = 3, 5
    WT = rng.standard_normal((nlf, nlf, nw)) * 10 + 1j * rng.standard_normal((nlf, nlf, nw))
    p = str(tmp_path / "W_Q1")
    rpa.write_wt(p, WT, domega=0.02)
    lines = open(p).read().splitlines()
    vals = []
    for iG in range(nlf):
        for jG in range(nlf):
            w = WT[jG, iG, 0]                # first frequency of Fortran WT(io, iG, jG)
            vals += [fortran_f(w.real, 15, 5), fortran_f(w.imag, 15, 5)]
    body = ["".join(vals[i:i + 10]) for i in range(0, len(vals), 10)]
    assert lines[0].split()[0] == "omega=" and float(lines[0].split()[1]) == 0.0
    assert lines[1:] == body
