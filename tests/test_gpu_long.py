"""The configured workloads for their whole length against the reference binary's own runs.

Fixtures (tests/golden/make_golden_long.py): the reference solver run on
  * the 400x40 Mach 0.1 channel for 1000 steps,
  * the 1200x120 Mach 2.43 channel for 4000 steps,
  * the 512x256 Rayleigh-Benard box for its steps (long_rayleigh_benard.json),
  * an 80x8 channel with the time-dependent inflow ramp (SIMPLE_TS_MPI.cpp:8102-8144),
  * the 2048x256 channel with the square at Mach 0.1, 0.5, 1.0 and 2.43 for 1000 steps,
each saving ten times into files of its own and logging every step.  The FP64 drop-in run must
write every one of those files byte for byte (the time loop SIMPLE_TS_MPI.cpp:3230-4691 for
the whole run).  The FP32-correction paths (precision 2 and 3) are then run for the same steps
and their per-field relative L2 distance from the FP64 fields is printed and bounded.  The
64-case batch (config 4) runs its 2000 steps as one batch against the reference's run of every
case alone.
"""
import json
import os
import tempfile

import numpy as np
import pytest

import sts_cases as sc
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

LONG = ["channel_inflow_ramp", "channel_ma0.1", "channel_ma2.43", "rayleigh_benard", "channel_2048_ma0.1",
        "channel_2048_ma0.5", "channel_2048_ma1.0", "channel_2048_ma2.43"]
FIELDS = ("u", "v", "p", "T", "rho")


def record(name):
    with open(os.path.join(GOLDEN, f"long_{name}.json")) as f:
        rec = json.load(f)
    arrays = dict(np.load(os.path.join(GOLDEN, f"long_{name}.npz")))
    return rec, arrays


def case_of(rec):
    from make_golden_long import long_case
    return long_case(rec["name"], rec["steps"])


def rel_l2(a, b, mask):
    d = np.linalg.norm((a - b)[mask])
    n = np.linalg.norm(b[mask])
    return float(d / n) if n > 0 else float(d)


@pytest.mark.parametrize("name", LONG)
def test_full_length_dropin_matches_reference(name, lib_built):
    """Every dump of every save, Tmp.txt and Iterations_in_loops.txt equal the reference's."""
    import sts
    from make_golden_long import file_digest
    rec, arrays = record(name)
    case = case_of(rec)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        sts.run_case(d, fixed_sweeps=False)
        lines = open(os.path.join(d, "Iterations_in_loops.txt")).read().split("\n")
        sweeps = np.array([int(l.split()[-1]) for l in lines if l.strip() and not l.startswith("it")])
        np.testing.assert_array_equal(sweeps, arrays["sweeps"], err_msg="sweep count per step")
        s = rec["stride"]
        for f in ("u", "v", "p", "Temper"):
            a = sc.read_field(d, f, rec["Nx"], rec["Ny"])[::s, ::s]
            np.testing.assert_array_equal(a, arrays[f], err_msg=f)
        bad = [f for f, h in rec["files"].items()
               if not os.path.exists(os.path.join(d, f)) or file_digest(os.path.join(d, f)) != h]
        assert not bad, f"files that differ from the reference's: {bad}"


def run_fields(case, rec, precision):
    """Steps the case in a fresh directory with the fixture's save cadence (a save applies the
    reference's output-time wall-temperature overwrite to the live state, so the saves are part
    of the trajectory); returns the final fields and the fluid mask."""
    import sts
    steps, every = rec["steps"], rec["save_every"]
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        fluid = sc.read_field(d, "vol_inf_fb", rec["Nx"], rec["Ny"]) == 0
        with sts.Solver(d, fixed_sweeps=False, precision=precision) as g:
            done = 0
            while done < steps:
                n = g.step(min(every, steps - done))
                assert n > 0
                done += n
                if done % every == 0:
                    g.write_outputs()
            return {f: g.field(f) for f in FIELDS}, fluid


# bounds of the FP32-correction paths' relative L2 distance from the FP64 fields after the whole
# run (measured on GB300: at most 4.4e-10 on the channel after 4000 steps, 6.5e-8 on the box after
# 20000 steps, where u is about 1e-5 of v)
BOUNDS = {"channel_ma2.43": 1e-8, "rayleigh_benard": 1e-6}


@pytest.mark.parametrize("name", ["channel_ma2.43", "rayleigh_benard"])
def test_full_length_fp32_corrections_error(name, lib_built):
    """Per-field relative L2 of precision 2 (FP32 sweeps on corrections, FP64 base fields,
    FP64 stopping residuals) and precision 3 (the same with double-float FP64 parts) against
    the FP64 path, which equals the reference on the sampled cells, after the whole run."""
    rec, arrays = record(name)
    case = case_of(rec)
    ref, fluid = run_fields(case, rec, 0)
    s = rec["stride"]
    sampled_fluid = arrays["vol_inf_fb"] == 0
    for f, g in (("u", "u"), ("v", "v"), ("p", "p"), ("T", "Temper")):
        # compared on fluid cells: the dump's wall cells hold the output-time overwrite
        np.testing.assert_array_equal(ref[f][::s, ::s][sampled_fluid], arrays[g][sampled_fluid], err_msg=f)
    out = {}
    for prec in (2, 3):
        got, _ = run_fields(case, rec, prec)
        out[prec] = {f: rel_l2(got[f], ref[f], fluid) for f in FIELDS}
    print(f"\nFP32_CORRECTIONS_ERROR {name} steps={rec['steps']} " + json.dumps(out))
    for prec, errs in out.items():
        for f, e in errs.items():
            assert e <= BOUNDS[name], (prec, f, e)


def test_batch64_full_length_matches_reference(lib_built):
    """The 64 cases of config 4 advanced together for their 2000 steps: every case's sweep count of
    every step and its final dumps equal the reference's run of that case alone (the reference
    saves at its last step and again after the loop, so the batch case saves twice)."""
    import sts
    from make_golden_long import file_digest, long_case
    with open(os.path.join(GOLDEN, "long_batch64.json")) as f:
        recs = json.load(f)
    arrays = np.load(os.path.join(GOLDEN, "long_batch64.npz"))
    with tempfile.TemporaryDirectory() as root:
        dirs = []
        for k in range(64):
            d = os.path.join(root, f"c{k:02d}")
            os.makedirs(d)
            long_case(f"batch64_{k}", recs[k]["steps"]).write(d)
            dirs.append(d)
        b = sts.Batch(dirs, fixed_sweeps=False)
        steps = recs[0]["steps"]
        assert b.step(steps) == steps
        bad = []
        for k, c in enumerate(b.cases):
            np.testing.assert_array_equal(c.sweep_history()[-steps:], arrays[f"{k}_sweeps"], err_msg=f"case {k}")
            c.write_outputs()
            c.write_outputs()
            for f in ("u.bin", "v.bin", "p.bin", "Temper.bin"):
                if file_digest(os.path.join(dirs[k], f)) != recs[k]["files"][f]:
                    bad.append((k, f))
        b.close()
        assert not bad, f"dumps that differ from the reference's: {bad}"
