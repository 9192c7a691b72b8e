"""warm_start 5: the learned stencil's start corrected on a window at the moving front by the U-Net
(BF16 tcgen05 kernels), trained on the GPU on step pairs the solver itself produces.

* With the network switched off, warm_start 5 is warm_start 4 bit for bit (the network's kernels
  only store training pairs), in graph and launch modes.
* Trained on the supersonic channel's own pairs, the network's loss falls; switched on, the run
  still converges to the same tolerance (fields within the tolerance-level distance of the cold
  start), and the sweep counts of the stencil alone and of the stencil with the network are
  printed side by side over the same steps.  The correction of p is gated (applied on a step's
  window only where, on the window completed last, it had lowered the stencil's largest error),
  so it adds sweeps rarely; T's correction is not applied.
"""
import tempfile

import numpy as np
import pytest

import sts_cases as sc

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "p", "T", "rho")


@pytest.mark.parametrize("use_graph", [True, False], ids=["graph", "launches"])
def test_network_off_equals_stencil(use_graph, lib_built):
    import sts
    case = sc.config_case("channel_ma2.43", scale=0.25, Nt=40)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        a = sts.Solver(d, fixed_sweeps=False, use_graph=use_graph, warm_start=4, precision=sts.MIXED)
        b = sts.Solver(d, fixed_sweeps=False, use_graph=use_graph, warm_start=5, precision=sts.MIXED)
        assert a.step(30) == 30 and b.step(30) == 30
        for f in FIELDS:
            np.testing.assert_array_equal(a.field(f), b.field(f), err_msg=f)
        np.testing.assert_array_equal(a.sweep_history(), b.sweep_history())
        info = b.warm_net_info()
        assert info["pairs"] == 29 and info["window"] == (32, 256)
        a.close()
        b.close()


def test_network_trains_on_solver_pairs_and_keeps_tolerance(lib_built, oracle_built):
    import ora
    import sts
    case = sc.config_case("channel_ma2.43", scale=0.5, Nt=200)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        cold = ora.Oracle(d, fixed_sweeps=False)
        cold.step(120)
        stencil = sts.Solver(d, fixed_sweeps=False, warm_start=4, precision=sts.MIXED)
        stencil.step(120)
        net = sts.Solver(d, fixed_sweeps=False, warm_start=5, precision=sts.MIXED)
        net.step(80)
        before, zero = net.warm_net_eval()
        net.warm_net_train(400, 3e-4)
        after, _ = net.warm_net_eval()
        net.warm_net_enable(True)
        net.step(40)
        s4 = stencil.sweep_history()[80:120]
        s5 = net.sweep_history()[80:120]
        print(f"loss on the stored pairs: zero correction {zero:.4g}, network {before:.4g} -> {after:.4g}; "
              f"sweeps per step over steps 81-120: "
              f"stencil {s4.mean():.3f}, stencil + network {s5.mean():.3f}, cold {cold.sweeps()[80:120].mean():.3f}")
        assert after < before and after < zero
        gate = net.warm_net_gate()  # the steps whose window took the correction (p only)
        print(f"steps with the network's correction of p: {gate['p']} of 40")
        assert 0 <= gate["p"] <= 40 and gate["T"] == 0
        assert s5.mean() <= s4.mean() + 0.25  # the gate keeps corrections that add sweeps rare
        for f in ("p", "T"):
            e = np.linalg.norm(net.field(f) - cold.field(f)) / np.linalg.norm(cold.field(f))
            assert e < 1e-6, (f, e)
        stencil.close()
        net.close()
