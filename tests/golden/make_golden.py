"""Generates the golden fixtures in tests/golden/ by running the reference solver itself.

The reference binary is compiled from the reference sources (oracle/build_oracle.py,
serial build with and without FIXED_NUMBER_OF_ITERATIONS_LOOP_3) and run on case
directories written by sts_cases.py.  For each case the fixture keeps, after the
run: the four field dumps u, v, p, Temper (in full for small meshes, as SHA-256 of
the raw little-endian bytes otherwise), vol_inf_fb, the sweep count of every step
(Iterations_in_loops.txt) and Tmp.txt, and the SHA-256 of every file the run writes into the
case directory (mesh files, drag-coefficient and pressure-control logs, continuity dumps ...)
except EnteredData.txt, whose rewrite records the wall-clock time.

Run from the repository root:  python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import shutil
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [os.path.join(ROOT, "simple-ts_gb300"), os.path.join(ROOT, "oracle")]
import sts_cases as sc  # noqa: E402
from build_oracle import build_reference  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
SHIPPED = "/root/reference"


def cases():
    """(name, Case, fixed_sweeps)"""
    out = []
    out.append(("channel_ma0.1_80x8_resid", sc.channel_case("c", 80, 8, 0.1, 0.00194, 1e-3, 20), False))
    out.append(("channel_ma0.1_80x8_fixed", sc.channel_case("c", 80, 8, 0.1, 0.00194, 1e-3, 20, tol=None), True))
    out.append(("channel_ma2.43_60x12_resid", sc.channel_case("c", 60, 12, 2.43, 0.00283, 2.5e-4, 30), False))
    out.append(("rayleigh_benard_32x16_resid", sc.rayleigh_benard_case("rb", 32, 16, Nt=30), False))
    c = sc.channel_case("c", 120, 12, 0.5, 0.003, 1e-3, 25, square_x=3.0)
    c.circles = [sc.Circle(xc=6.0, yc=0.5, rc=0.18)]
    c.restart = sc.channel_initial_state(c, sc.inflow_velocity(0.5))
    out.append(("channel_circle_120x12_resid", c, False))
    out.append(("channel_ma0.1_400x40_resid_5steps", sc.config_case("channel_ma0.1", Nt=5), False))
    # the diagnostics of the time loop: drag coefficients of every body every 2 steps, the
    # short-format summary and the continuity residual dumps (binary and text)
    c = sc.channel_case("c", 80, 8, 0.3, 0.002, 1e-3, 6)
    c.entered.update(Nt_save_DragCoefficient=2, WriteDataInShortFormat_kind=1, ToSolveContinuityEquation=1)
    for P in c.polygons:
        P.drag = 1
    out.append(("channel_diagnostics_80x8_resid", c, False))
    c = sc.rayleigh_benard_case("rb", 32, 16, Nt=5)
    c.entered.update(ToSolveContinuityEquation=1, ToWriteSolvedDataToBinaryFile=0, Nt_save_DragCoefficient=3,
                     N_I_p_c=3)
    for P in c.polygons:
        P.drag = 1
    out.append(("rayleigh_benard_diagnostics_txt_32x16_fixed", c, True))
    # periodic saves that each keep their own copy (ToWriteSolvedDataToNewFiles): every dump of
    # every save is a file of its own, named by the time of the save; binary with the continuity
    # dumps of every step, and text
    c = sc.channel_case("c", 80, 8, 0.3, 0.002, 1e-3, 8)
    c.entered.update(Nt_save_solved_data=2, ToWriteSolvedDataToNewFiles=1, ToSolveContinuityEquation=1)
    out.append(("channel_newfiles_80x8_resid", c, False))
    c = sc.rayleigh_benard_case("rb", 32, 16, Nt=4)
    c.entered.update(Nt_save_solved_data=1, ToWriteSolvedDataToNewFiles=1, ToWriteSolvedDataToBinaryFile=0,
                     N_I_p_c=3)
    out.append(("rayleigh_benard_newfiles_txt_32x16_fixed", c, True))
    return out




def file_digest(path):
    """SHA-256 of a file; in text files the sign of a printed NaN ("-nan" on x86, "nan" on Arm:
    the host CPU's default NaN) is normalised away, keeping the field width of setw columns."""
    data = open(path, "rb").read()
    if path.endswith(".txt"):
        data = data.replace(b"-nan", b" nan")
    return hashlib.sha256(data).hexdigest()


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).astype(a.dtype.newbyteorder("<")).tobytes()).hexdigest()


def run_one(name, case, fixed, exe, copy_files=()):
    d = tempfile.mkdtemp(prefix="golden_")
    try:
        case.entered["Nt_save_temp_data"] = 1  # one log line per step
        case.write(d)
        for f in copy_files:
            shutil.copy(f, d)
        import subprocess
        before = {f: hashlib.sha256(open(os.path.join(d, f), "rb").read()).hexdigest() for f in os.listdir(d)}
        subprocess.run([exe], cwd=d, capture_output=True, check=True)
        e = sc.read_entered_data(os.path.join(d, "EnteredData.txt"))
        Nx, Ny = int(e["Nx"]), int(e["Ny"])
        rec = {"name": name, "Nx": Nx, "Ny": Ny, "fixed_sweeps": bool(fixed), "steps": int(case.entered["Nt"])}
        arrays = {}
        for f in ("u", "v", "p", "Temper", "vol_inf_fb"):
            a = sc.read_field(d, f, Nx, Ny)
            rec["sha256_" + f] = digest(a)
            arrays[f] = a
        lines = open(os.path.join(d, "Iterations_in_loops.txt")).read().split("\n")
        rec["sweeps"] = [int(l.split()[-1]) for l in lines if l.strip() and not l.startswith("it")]
        rec["tmp_txt"] = open(os.path.join(d, "Tmp.txt")).read()
        after = {f: file_digest(os.path.join(d, f)) for f in os.listdir(d)}
        rec["files"] = {f: h for f, h in sorted(after.items())
                        if f != "EnteredData.txt" and before.get(f) != h}  # what the run wrote
        small = Nx * Ny <= 4000
        if small:
            np.savez_compressed(os.path.join(OUT, name + ".npz"), **arrays)
        rec["arrays"] = small
        return rec
    finally:
        shutil.rmtree(d, ignore_errors=True)


def main():
    exes = build_reference()
    if exes is None:
        raise SystemExit("the reference sources are not present; fixtures cannot be regenerated here")
    records = []
    for name, case, fixed in cases():
        exe = exes["simple_ts_fixed"] if fixed else exes["simple_ts_resid"]
        records.append(run_one(name, case, fixed, exe))
        print(name, records[-1]["Nx"], records[-1]["Ny"], records[-1]["sweeps"][:8])
    # the example input shipped with the reference, run from its own files and from the
    # restatement in sts_cases.shipped_example(): both runs must agree byte for byte
    if os.path.exists(os.path.join(SHIPPED, "EnteredData.txt")):
        e = sc.read_entered_data(os.path.join(SHIPPED, "EnteredData.txt"))
        e.update(Nt=5, Nt_save_solved_data=5, Nt_save_temp_data=1)
        orig = run_one("shipped_example_5steps", sc.Case("shipped", e), True, exes["simple_ts_fixed"],
                       [os.path.join(SHIPPED, "solve_polyhedrons_b.txt")])
        mine = run_one("shipped_example_5steps", sc.shipped_example(5), True, exes["simple_ts_fixed"])
        for k in orig:
            if k.startswith("sha256") or k in ("sweeps", "files"):
                assert orig[k] == mine[k], ("restated example differs from the shipped files", k)
        records.append(mine)
        print(mine["name"], mine["Nx"], mine["Ny"], mine["sweeps"])
    with open(os.path.join(OUT, "golden.json"), "w") as f:
        json.dump(records, f, indent=1)


if __name__ == "__main__":
    main()
