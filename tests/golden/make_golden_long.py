"""Generates the full-length golden fixtures (tests/golden/long_*.json, long_*.npz) by running
the reference solver itself on the configured workloads for their whole length.

Cases (FP64, the reference's tolerance-terminated sweep loop at 1e-8, cold start):
  * channel_ma0.1   -- 400x40 channel past a square, Mach 0.1, Kn 0.00194, dt 1e-3, 1000 steps;
  * channel_ma2.43  -- 1200x120 supersonic channel, Mach 2.43, Kn 0.00283, dt 2.5e-4, 4000 steps;
  * rayleigh_benard -- 512x256 periodic Rayleigh-Benard box, Kn 0.01, g = 1, dt 5e-5, seeded
                       noise; as many steps as given on the command line (20000 by default).
  * channel_inflow_ramp -- an 80x8 channel whose inflow speed follows the reference's
                       time-dependent inflow (use_interpolation_for_u_BC_by_time,
                       SIMPLE_TS_MPI.cpp:8102-8144), 40 steps, dumps in full;
  * channel_2048_ma<M> -- the 2048x256 channel with the square at Mach M (Kn 0.003, dt 1.25e-4),
                       1000 steps by default;
  * batch64_<k>     -- case k of the 64-case batch (seed 20261204) for its 2000 steps, the final
                       dumps only (one save at the end).

Every case saves ten times during the run into files of their own
(ToWriteSolvedDataToNewFiles, SIMPLE_TS_MPI.cpp:5607-5631) and writes a log line every step,
so the fixture holds the SHA-256 of every dump of every save, of Tmp.txt and of
Iterations_in_loops.txt, the sweep count of every step, and the final u, v, p, T on every
eighth cell in x and y (for a relative L2 distance of runs that are not bit-exact).  The
reference binary is built by oracle/build_oracle.py from the reference sources.

Run from the repository root, one case per process (they are independent):
  python tests/golden/make_golden_long.py channel_ma0.1
  python tests/golden/make_golden_long.py rayleigh_benard 20000
  python tests/golden/make_golden_long.py batch64_17          (then: ... make_golden_long.py --merge-batch)
The 64 batch cases are merged into long_batch64.json / long_batch64.npz by --merge-batch.
"""
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [os.path.join(ROOT, "simple-ts_gb300"), os.path.join(ROOT, "oracle")]
import sts_cases as sc  # noqa: E402
from build_oracle import build_reference  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
STRIDE = 8  # sampled cells: every STRIDE-th in x and in y


def long_case(name, steps=None):
    """The Case of a long fixture, with its save cadence set (ten saves, a log line every step)."""
    if name.startswith("batch64_"):  # one case of the 64-case batch (seed 20261204), final dumps only
        k = int(name[len("batch64_"):])
        c = sc.batch_cases(n=64, Nt=steps or 2000)[k]
        c.entered.update(Nt_save_solved_data=int(c.entered["Nt"]), Nt_save_temp_data=1)
        return c
    if name == "channel_inflow_ramp":
        c = sc.channel_case("c", 80, 8, 0.3, 0.002, 1e-3, steps or 40)
        c.entered.update(use_interpolation_for_u_BC_by_time=1, t_BC_b=0.005, t_BC_e=0.025,
                         u_BC_xb_t_BC_b=sc.inflow_velocity(0.3), u_BC_xb_t_BC_e=sc.inflow_velocity(0.6))
    else:
        c = sc.config_case(name, Nt=steps)
    Nt = int(c.entered["Nt"])
    c.entered.update(Nt_save_solved_data=max(Nt // 10, 1), ToWriteSolvedDataToNewFiles=1, Nt_save_temp_data=1)
    return c


def sample(a):
    return np.ascontiguousarray(a[::STRIDE, ::STRIDE])


def file_digest(path):
    """SHA-256 of a file; a printed NaN's sign (x86 "-nan", Arm "nan") is normalised in text files."""
    data = open(path, "rb").read()
    if path.endswith(".txt"):
        data = data.replace(b"-nan", b" nan")
    return hashlib.sha256(data).hexdigest()


def merge_batch():
    """long_batch64_<k>.{json,npz} (k = 0..63) into long_batch64.json (records by case) and
    long_batch64.npz (arrays named <k>_<field>); the per-case files are removed."""
    recs, arrays = [], {}
    for k in range(64):
        base = os.path.join(OUT, f"long_batch64_{k}")
        with open(base + ".json") as f:
            recs.append(json.load(f))
        for key, a in np.load(base + ".npz").items():
            arrays[f"{k}_{key}"] = a
    with open(os.path.join(OUT, "long_batch64.json"), "w") as f:
        json.dump(recs, f, indent=1)
    np.savez_compressed(os.path.join(OUT, "long_batch64.npz"), **arrays)
    for k in range(64):
        for ext in (".json", ".npz"):
            os.remove(os.path.join(OUT, f"long_batch64_{k}{ext}"))


def main():
    if sys.argv[1] == "--merge-batch":
        return merge_batch()
    name = sys.argv[1]
    steps = int(sys.argv[2]) if len(sys.argv) > 2 else None
    exes = build_reference()
    if exes is None:
        raise SystemExit("the reference sources are not present; fixtures cannot be regenerated here")
    case = long_case(name, steps)
    d = tempfile.mkdtemp(prefix="golden_long_")
    try:
        case.write(d)
        before = {f: file_digest(os.path.join(d, f)) for f in os.listdir(d)}
        t0 = time.time()
        subprocess.run([exes["simple_ts_resid"]], cwd=d, capture_output=True, check=True)
        wall = time.time() - t0
        e = sc.read_entered_data(os.path.join(d, "EnteredData.txt"))
        Nx, Ny = int(e["Nx"]), int(e["Ny"])
        after = {f: file_digest(os.path.join(d, f)) for f in os.listdir(d)}
        files = {f: h for f, h in sorted(after.items()) if f != "EnteredData.txt" and before.get(f) != h}
        lines = open(os.path.join(d, "Iterations_in_loops.txt")).read().split("\n")
        sweeps = np.array([int(l.split()[-1]) for l in lines if l.strip() and not l.startswith("it")], np.uint16)
        arrays = {"sweeps": sweeps}
        for f in ("u", "v", "p", "Temper", "vol_inf_fb"):
            arrays[f] = sample(sc.read_field(d, f, Nx, Ny))
        np.savez_compressed(os.path.join(OUT, f"long_{name}.npz"), **arrays)
        rec = {"name": name, "Nx": Nx, "Ny": Ny, "steps": int(case.entered["Nt"]),
               "save_every": int(case.entered["Nt_save_solved_data"]), "stride": STRIDE,
               "reference_wall_s": round(wall, 1), "files": files}
        with open(os.path.join(OUT, f"long_{name}.json"), "w") as f:
            json.dump(rec, f, indent=1)
        print(name, Nx, Ny, len(sweeps), "steps", f"{wall:.0f} s", "mean sweeps", sweeps.mean())
    finally:
        shutil.rmtree(d, ignore_errors=True)


if __name__ == "__main__":
    main()
