"""Global FP64 conservation sums on the device (mass, momentum, internal and kinetic energy over the
fluid cells), in a fixed summation order: equal bit for bit to the oracle's sums of the same state."""
import tempfile

import numpy as np
import pytest

import sts_cases as sc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", ["channel", "rayleigh_benard", "batch"])
def test_conservation_sums_match_oracle(which, lib_built, oracle_built):
    import ora
    import sts
    if which == "channel":
        case = sc.channel_case("c", 150, 15, 2.43, 0.00283, 2.5e-4, 50)
    else:
        case = sc.rayleigh_benard_case("rb", 64, 32, Nt=50)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        o = ora.Oracle(d, fixed_sweeps=False)
        if which == "batch":
            b = sts.Batch([d, d], fixed_sweeps=False)
            g = b.cases[1]
        else:
            g = sts.Solver(d, fixed_sweeps=False)
        np.testing.assert_array_equal(g.conservation(), o.conservation())
        for k in range(3):
            if which == "batch":
                b.step(4)
            else:
                g.step(4)
            o.step(4)
            np.testing.assert_array_equal(g.conservation(), o.conservation(), err_msg=f"after {4 * (k + 1)} steps")
        if which == "batch":
            b.close()
        else:
            g.close()
