"""The tcgen05 GEMM block of the photon guide's network (fr_tc.cuh) against a
host GEMM on the same BF16 inputs: FP32 accumulation, so errors stay at the
FP32 rounding of 64-term sums of products of magnitude <= 1."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('seed', [1, 2, 3])
def test_tcgen05_gemm_matches_host(seed):
    from frsppm import abi
    err = abi.check_tc_gemm(seed)
    assert (err < 1e-4).all(), err
