"""The oracle's warm starts on the CPU: the convolutional predictor (warm_start 4) takes fewer
sweeps than quadratic extrapolation on a moving front, and its runs stay within the
tolerance-level distance of the cold start."""
import tempfile

import numpy as np

import sts_cases as sc


def test_conv_predictor_beats_extrapolation(oracle_built):
    import ora
    case = sc.config_case("channel_ma2.43", scale=0.5, Nt=60)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        runs = {}
        for warm in (0, 2, 4):
            o = ora.Oracle(d, fixed_sweeps=False, warm_start=warm)
            assert o.step(60) == 60
            runs[warm] = (o.sweeps()[20:60].mean(), o.field("p"), o.field("T"))
        print({w: r[0] for w, r in runs.items()})
        assert runs[4][0] < runs[2][0] < runs[0][0]
        for k, f in ((1, "p"), (2, "T")):
            e = np.linalg.norm(runs[4][k] - runs[0][k]) / np.linalg.norm(runs[0][k])
            assert e < 1e-6, (f, e)
