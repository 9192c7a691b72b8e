"""The FP64 kernels divide by mesh sums, ht, 3 and the sweep's loop-invariant T denominator
through correctly rounded reciprocals (Markstein's method).  Bit-exact parity with the
reference needs every such quotient to equal the IEEE quotient bit for bit."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 20261203, 0xDEADBEEF])
def test_reciprocal_division_matches_ieee(seed, lib_built):
    import sts
    assert sts.check_division(1 << 28, seed) == 0
