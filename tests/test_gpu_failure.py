"""Failure detection without a GPU fault: the sweep loops' grid barrier waits a bounded number of
polls, and a wait that runs out ends the launch with a status the host reads (STS_ERR_TIMEOUT),
leaving the device usable.  The wait is made to run out by a CTA that never arrives."""
import pytest

pytestmark = pytest.mark.gpu


def test_barrier_completes_when_every_cta_arrives(lib_built):
    import sts
    assert sts.check_barrier_timeout(skip_cta=-1, spin_limit=1 << 20, rounds=200) == sts.STS_OK


@pytest.mark.parametrize("skip", [0, 5])
def test_barrier_wait_gives_up_with_timeout_status(skip, lib_built):
    import sts
    assert sts.check_barrier_timeout(skip_cta=skip, spin_limit=1 << 12, rounds=3) == sts.STS_ERR_TIMEOUT
    # the device is still usable: a full barrier run afterwards completes
    assert sts.check_barrier_timeout(skip_cta=-1, spin_limit=1 << 20, rounds=10) == sts.STS_OK


def test_timeout_code_is_distinct(lib_built):
    import sts
    codes = {sts.STS_ERR_ARG, sts.STS_ERR_INPUT, sts.STS_ERR_CUDA, sts.STS_ERR_NONFINITE, sts.STS_ERR_TIMEOUT}
    assert len(codes) == 5
