"""GPU: tcgen05 building blocks (descriptors, swizzle, TMEM read-back)."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", [0, 1, 2])
def test_umma_gemm_matches_cuda_core_product(rpa, which):
    err = rpa.selftest(which)
    assert err < 1e-5, err
