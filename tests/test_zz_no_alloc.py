"""GPU: the allocation-free Dyson entry point against rpa_dyson.

rpa_dyson_noalloc serves callers that cannot allocate device memory when they
need the solve (a host framework that owns all device allocations, or serving
code that cannot pay for cudaMalloc's device synchronisation per request).  It
runs with a fixed workspace compiled into the library.  This file is collected
last on purpose, so a failure here cannot hide the result of any other test.
The check runs two calls in a row on the same device buffers, since every call
reuses the same workspace.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_DYSON = 1e-9  # as in test_gpu_parity.py


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _chi_and_refs(s, rpa, orc):
    """chi0 of the plain FP64 path for system s, rpa_dyson's W and eps^-1_00 on
    it, and the oracle's Dyson restatement (gjel, genWT) of the same chi0."""
    ctx = rpa.Context()
    ctx.load_system(s)
    ctx.chi0(rpa.MODE_CHARGE, want=False, **rpa.sloss_args(s))
    chi = ctx.kk(rpa.KK_SLOSS_REAL)                 # numpy (jG, iG, io) == Fortran chi0(io, iG, jG)
    WT_ref, _, head_ref = ctx.dyson(s.c0, s.cfg.eps)
    ctx.close()
    V = orc.genV(s)                                  # numpy (jG, iG) == V(iG, jG): column-major already
    WT_o, Ei_o, rc = orc.dyson(chi, V, fast_wt=True)
    assert rc == 0
    return chi, V, (WT_ref, head_ref), (WT_o, Ei_o[0, 0, :])


def _noalloc(rpa, chi, V, calls, wait):
    """Calls rpa_dyson_noalloc `calls` times in a row on the same device
    buffers; wait=False passes n_singular = NULL (no wait inside the call)."""
    import torch
    n, nwo = chi.shape[0], chi.shape[2]
    # device layout: [io][iG + n*jG]
    chi_dev = torch.from_numpy(np.ascontiguousarray(np.transpose(chi, (2, 0, 1))).view(np.float64)).cuda()
    V_dev = torch.from_numpy(np.ascontiguousarray(V)).cuda()
    L = rpa.load_library()
    stream = torch.cuda.current_stream().cuda_stream
    out = []
    for _ in range(calls):
        WT_dev = torch.full((nwo, n, n, 2), float("nan"), dtype=torch.float64, device="cuda")
        head_dev = torch.full((nwo, 2), float("nan"), dtype=torch.float64, device="cuda")
        nsing = C.c_int(-1)
        rc = L.rpa_dyson_noalloc(chi_dev.data_ptr(), V_dev.data_ptr(), n, nwo, WT_dev.data_ptr(),
                                 head_dev.data_ptr(), stream, C.byref(nsing) if wait else None)
        assert rc == rpa.RPA_OK
        if wait:
            assert nsing.value == 0
        torch.cuda.synchronize()
        WT = WT_dev.cpu().numpy().view(np.complex128)[..., 0]   # [io, jG, iG]
        head = head_dev.cpu().numpy().view(np.complex128)[:, 0]
        out.append((np.transpose(WT, (1, 2, 0)), head))
    return out


def test_noalloc_dyson_matches_rpa_dyson_twice(synth, rpa, orc):
    """Two calls in a row (NGloc 19, 200 frequencies): W and eps^-1_00 equal
    rpa_dyson's and the oracle's Dyson of the same chi0."""
    s = synth.build(synth.config_grid24())
    chi, V, (WT_ref, head_ref), (WT_o, head_o) = _chi_and_refs(s, rpa, orc)
    for call, (WT, head) in enumerate(_noalloc(rpa, chi, V, 2, True)):
        assert rel(WT, WT_ref) < TOL_DYSON, call
        assert rel(head, head_ref) < TOL_DYSON, call
        assert rel(WT, WT_o) < TOL_DYSON, call
        assert rel(head, head_o) < TOL_DYSON, call


def test_noalloc_dyson_at_the_size_limit(synth, rpa, orc):
    """n = 96, the largest size the workspace holds, with 40 frequencies, so
    all 32 blocks run and the last block's workspace ends at the array's end;
    the second call passes n_singular = NULL (no wait inside the call)."""
    s = synth.build(synth.config_small(nlf=96, lf="xyz", npw=200, no=41))
    chi, V, (WT_ref, head_ref), (WT_o, head_o) = _chi_and_refs(s, rpa, orc)
    assert chi.shape[0] == 96 and chi.shape[2] >= 32
    res = _noalloc(rpa, chi, V, 1, True) + _noalloc(rpa, chi, V, 1, False)
    for call, (WT, head) in enumerate(res):
        assert rel(WT, WT_ref) < TOL_DYSON, call
        assert rel(head, head_ref) < TOL_DYSON, call
        assert rel(WT, WT_o) < TOL_DYSON, call
        assert rel(head, head_o) < TOL_DYSON, call


def test_noalloc_rejects_oversized_matrices(rpa):
    L = rpa.load_library()
    nsing = C.c_int(0)
    rc = L.rpa_dyson_noalloc(C.c_void_p(16), C.c_void_p(16), 97, 4, C.c_void_p(16), None, None, C.byref(nsing))
    assert rc == rpa.RPA_EINVAL
