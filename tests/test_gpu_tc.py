"""GPU: tcgen05 building blocks (descriptors, swizzle, TMEM read-back)."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", [0, 1, 2])
def test_umma_gemm_matches_cuda_core_product(rpa, which):
    err = rpa.selftest(which)
    assert err < 1e-5, err


def test_bounded_wait_times_out_and_the_device_stays_usable(rpa):
    """A device wait whose flag nothing sets gives up, the host reads
    RPA_ETIMEOUT, and the next tensor-core self-test still passes."""
    import ctypes as C
    L = rpa.load_library()
    cycles = C.c_double()
    assert L.rpa_selftest(3, C.byref(cycles)) == rpa.RPA_ETIMEOUT
    assert cycles.value > 0
    assert rpa.selftest(0) < 1e-5


def test_umma_with_a_in_tensor_memory(rpa):
    """tcgen05.mma with A in TMEM (rows in lanes, two f16 of K per column)."""
    assert rpa.selftest(4) < 1e-5
