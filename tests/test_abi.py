"""CPU checks of the C ABI: the library builds for sm_103a, loads, exports
every entry point of include/rpa_gpu.h, and its host-only parts (init_igk,
the KK kernel matrix) agree with the oracle.  No kernel runs here."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "rpa_gpu.h")


def header_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(rpa_\w+)\s*\(", txt, re.M)))


def test_every_declared_symbol_is_exported(rpa):
    L = rpa.load_library()
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    assert sorted(rpa.EXPORTS) == names


def test_create_fails_loudly_without_a_device(rpa):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(rpa.RpaError) as e:
        rpa.Context()
    assert e.value.code == rpa.RPA_ECUDA


def test_kk_matrix_matches_oracle_loops(rpa, orc, npo):
    rng = np.random.default_rng(0)
    for no in (3, 4, 5, 9, 40):
        dw = 0.013
        Ks = rpa.kk_matrix(rpa.KK_SLOSS_REAL, no, dw)
        assert np.allclose(Ks, npo.kk_matrix_sloss(no, dw), rtol=1e-15, atol=0)
        S = rng.standard_normal((3, 3, no))
        chi = orc.kk_sloss(S, dw)
        re = np.einsum("oj,baj->bao", Ks, S)
        assert np.abs(re - chi.real).max() < 1e-13 * np.abs(chi.real).max()
        Kc = rpa.kk_matrix(rpa.KK_OPTABS_COMPLEX, no, dw)
        Sc = rng.standard_normal((2, 2, 2 * no + 1)) + 1j * rng.standard_normal((2, 2, 2 * no + 1))
        chic = orc.kk_optabs(Sc, dw)
        prod = np.einsum("oj,baj->bao", Kc, Sc)
        srow = Sc[:, :, no: 2 * no - 1]            # S0(io-1), io = 1..no-1
        got = prod - 1j * np.pi * srow
        assert np.abs(got - chic).max() < 1e-13 * np.abs(chic).max()


def test_sloss_kk_keeps_else_if_semantics(rpa):
    """Sloss' else-if chain never applies the end-point overrides away from
    jo == io, unlike Optabs (Sloss.f90:979-1040 vs Optabs.f90:1145-1208)."""
    no, dw = 12, 0.1
    K = rpa.kk_matrix(rpa.KK_SLOSS_REAL, no, dw)
    io = 5
    oi, oj = (io - 1) * dw, (np.arange(no)) * dw
    want = np.where(np.arange(1, no + 1) != io, dw / np.where(oi != oj, oi - oj, 1.0), 0.0)
    fp = dw / (oi + oj)
    fp[0] *= 0.5
    fp[-1] *= 0.5
    assert np.allclose(K[io - 1], want - fp, rtol=1e-15, atol=0)
