"""TEST INFRASTRUCTURE: the reference solver's own MPI build on the host cores of this machine.

The build (oracle/build_oracle.py build_reference_mpi) links the reference with the minimal
shared-memory MPI of oracle/mpishim; `run(case_dir, n)` runs it as the reference's MPI jobs are
run, in two passes: with ToOnlyWriteDataFor_Nx_Ny_ForAllSubDomains_AndExit = 1 the reference writes
its own subdomain layout (Nx_Ny_ForAllSubDomains.txt, one strip per rank along x,
SIMPLE_TS_MPI.cpp:10745-10900) and exits, then the solve runs on n ranks (N_SubDomains_x = n).
Needs the reference sources, so it runs only where they are.

  python oracle/reference_mpi.py channel_ma2.43 8 40     # case, ranks, steps: cell-steps/s
"""
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def run(case, case_dir, n, timeout=3600):
    """Writes `case` (an sts_cases.Case) into case_dir for n ranks and runs the reference MPI build
    there; returns the solve's wall seconds (the layout pass excluded)."""
    from build_oracle import build_reference_mpi
    exes = build_reference_mpi()
    if exes is None:
        raise RuntimeError("the reference sources are not present")
    cmd = [exes["mpishim_run"], str(n), exes["simple_ts_mpi_resid"]]
    case.entered.update(N_SubDomains_x=n, N_SubDomains_y=1, ToOnlyWriteDataFor_Nx_Ny_ForAllSubDomains_AndExit=1)
    case.write(case_dir)
    subprocess.run(cmd, cwd=case_dir, capture_output=True, check=True, timeout=timeout)
    case.entered["ToOnlyWriteDataFor_Nx_Ny_ForAllSubDomains_AndExit"] = 0
    case.write(case_dir)
    t0 = time.perf_counter()
    subprocess.run(cmd, cwd=case_dir, capture_output=True, check=True, timeout=timeout)
    return time.perf_counter() - t0


def main():
    sys.path[:0] = [os.path.join(ROOT, "simple-ts_gb300"), HERE]
    import sts_cases as sc
    which, n, steps = sys.argv[1], int(sys.argv[2]), int(sys.argv[3])
    case = sc.config_case(which, Nt=steps)
    case.entered.update(Nt_save_temp_data=steps, Nt_save_solved_data=steps)
    with tempfile.TemporaryDirectory() as d:
        wall = run(case, d, n)
    print(f"{which} {case.Nx}x{case.Ny}, {n} ranks, {steps} steps: {wall:.2f} s, "
          f"{case.Nx * case.Ny * steps / wall:.3e} cell-steps/s (set-up included)")


if __name__ == "__main__":
    main()
