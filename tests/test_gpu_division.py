"""The FP64 kernels divide by mesh sums, ht, 3 and the sweep's loop-invariant T denominator
through correctly rounded reciprocals (Markstein's method).  Bit-exact parity with the
reference needs every such quotient to equal the IEEE quotient bit for bit."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 20261203, 0xDEADBEEF])
def test_reciprocal_division_matches_ieee(seed, lib_built):
    import sts
    assert sts.check_division(1 << 28, seed) == 0


def test_double_float_arithmetic_accuracy(lib_built):
    """Precision mode 3's double-float words carry about 47 bits: every basic operation must stay
    within a few units of 2^-47 of the FP64 result."""
    import sts
    err = sts.check_double_float(1 << 24, seed=3)
    print(err)
    for k, e in err.items():
        assert e < 2.0 ** -44, (k, e)


def test_fp64_rates(lib_built):
    """The FP64 throughput the bit-exact kernels' roofline is taken against: positive and within
    a plausible range for one GPU, with the fused multiply-add no slower than a plain add or
    multiply (one FP64 instruction each)."""
    import sts
    r = sts.fp64_rates()
    print(r)
    for k in ("add", "mul", "fma"):
        assert 10.0 < r[k] < 1.0e5, (k, r[k])
    assert r["fma"] > 0.8 * min(r["add"], r["mul"])
