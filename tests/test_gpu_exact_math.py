"""The kernels' float replacements for the reference's double-precision
expressions (fr_exact.cuh) against those expressions, on the device.

Each replacement evaluates in float-float arithmetic with an error bound and
returns a float only when the bound proves it is the double expression's
rounded result; otherwise it evaluates the double expression.  Over a billion
seeded inputs per function, inside and far outside the ranges the renderer
passes, every value the float path returns must equal the double result bit
for bit, and the float path must carry the bulk of the calls."""
import pytest

pytestmark = pytest.mark.gpu

SAMPLES = 1 << 30


def test_float_paths_equal_double_expressions():
    from frsppm import abi
    res = abi.check_exact_math(SAMPLES, seed=20261203)
    for name, (fast, mismatches) in res.items():
        assert mismatches == 0, (name, fast, mismatches)
        # Half of the inputs are drawn from the renderer's ranges, half from
        # wide ones that partly fall back to double by design.
        assert fast >= 0.4 * SAMPLES, (name, fast)


def test_seeds_differ():
    from frsppm import abi
    a = abi.check_exact_math(1 << 20, seed=1)
    b = abi.check_exact_math(1 << 20, seed=2)
    assert all(a[n][1] == 0 and b[n][1] == 0 for n in a)
    assert a != b
