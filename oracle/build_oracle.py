"""Build recipe for the CPU oracle (test infrastructure, not part of the product).

* ``oracle/_build/libsts_oracle.so`` and ``oracle/_build/sts_oracle``: the C++
  restatement in ``sts_oracle.cpp`` (always built; runs on x86 and on Arm).
* ``oracle/_ref/simple_ts_fixed`` and ``oracle/_ref/simple_ts_resid``: the
  reference solver itself, compiled from its own sources where they lie
  (``/root/reference``) when that tree exists.  The serial build switches off
  ``#define COMPILE_MPI`` (SIMPLE_TS_MPI.cpp:37); the residual build also
  switches off ``#define FIXED_NUMBER_OF_ITERATIONS_LOOP_3`` (SIMPLE_TS_MPI.cpp:56).
  The patch is applied on a pipe into the compiler; no copy of the sources is
  written anywhere.

Both use ``-ffp-contract=off`` so that no multiply-add is fused on Arm either.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE = "/root/reference"
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-w"]


def _newer(out, srcs):
    return os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs)


def build_oracle(force=False):
    src = os.path.join(HERE, "sts_oracle.cpp")
    bdir = os.path.join(HERE, "_build")
    os.makedirs(bdir, exist_ok=True)
    lib = os.path.join(bdir, "libsts_oracle.so")
    exe = os.path.join(bdir, "sts_oracle")
    procs = []
    if force or not _newer(lib, [src]):
        procs.append(subprocess.Popen(["g++"] + FLAGS + ["-fPIC", "-shared", src, "-o", lib]))
    if force or not _newer(exe, [src]):
        procs.append(subprocess.Popen(["g++"] + FLAGS + ["-DSTS_ORACLE_MAIN", src, "-o", exe]))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("oracle build failed")
    return lib, exe


def build_reference(force=False):
    """Compile the reference solver (serial) when its sources are present; returns paths or None."""
    main = os.path.join(REFERENCE, "SIMPLE_TS_MPI.cpp")
    if not os.path.exists(main):
        return None
    rdir = os.path.join(HERE, "_ref")
    os.makedirs(rdir, exist_ok=True)
    others = [os.path.join(REFERENCE, f) for f in
              ("Circles_Objects.cpp", "Polyhedrons_Objects.cpp", "Objects_for_Solving.cpp")]
    out = {}
    variants = {
        "simple_ts_fixed": [r"s|^#define COMPILE_MPI\r*$|/* serial build */|"],
        "simple_ts_resid": [r"s|^#define COMPILE_MPI\r*$|/* serial build */|",
                            r"s|^#define FIXED_NUMBER_OF_ITERATIONS_LOOP_3\r*$|/* residual-terminated */|"],
    }
    procs = []
    for name, seds in variants.items():
        exe = os.path.join(rdir, name)
        out[name] = exe
        if not force and _newer(exe, [main] + others):
            continue
        sed_args = " ".join(f"-e '{s}'" for s in seds)
        cmd = (f"sed {sed_args} {main} | g++ -O3 -msse2 -ffp-contract=off -w -I{REFERENCE} "
               f"-x c++ - -x none {' '.join(others)} -o {exe}")
        if os.uname().machine not in ("x86_64", "i686"):
            cmd = cmd.replace("-msse2 ", "")
        procs.append(subprocess.Popen(["bash", "-c", cmd]))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("reference build failed")
    return out


def build_reference_mpi(force=False):
    """The reference solver's own MPI build (COMPILE_MPI kept, residual-terminated sweeps) against the
    minimal shared-memory MPI of oracle/mpishim, and its launcher: oracle/_ref/simple_ts_mpi_resid
    and oracle/_ref/mpishim_run, when the reference sources are present (returns paths or None).
    Run as `mpishim_run N simple_ts_mpi_resid` in a case directory whose EnteredData.txt asks for N
    subdomains.  Compiled as C++98: the reference's global `rank` clashes with std::rank of C++11."""
    main = os.path.join(REFERENCE, "SIMPLE_TS_MPI.cpp")
    if not os.path.exists(main):
        return None
    rdir = os.path.join(HERE, "_ref")
    shim = os.path.join(HERE, "mpishim")
    os.makedirs(rdir, exist_ok=True)
    others = [os.path.join(REFERENCE, f) for f in
              ("Circles_Objects.cpp", "Polyhedrons_Objects.cpp", "Objects_for_Solving.cpp", "DomainDecomposition2D.cpp")]
    shim_src = [os.path.join(shim, f) for f in ("mpi.h", "mpishim.c", "mpishim_seg.h", "mpishim_run.c")]
    exe = os.path.join(rdir, "simple_ts_mpi_resid")
    run = os.path.join(rdir, "mpishim_run")
    procs = []
    if force or not _newer(exe, [main] + others + shim_src):
        obj = os.path.join(rdir, "mpishim.o")
        cmd = (f"gcc -O2 -c {os.path.join(shim, 'mpishim.c')} -o {obj} && "
               f"sed -e 's|^#define FIXED_NUMBER_OF_ITERATIONS_LOOP_3\r*$|/* residual-terminated */|' {main} | "
               f"g++ -std=gnu++98 -O3 -msse2 -ffp-contract=off -w -I{shim} -I{REFERENCE} -x c++ - -x none {' '.join(others)} "
               f"{obj} -o {exe} -lpthread -lrt")
        if os.uname().machine not in ("x86_64", "i686"):
            cmd = cmd.replace("-msse2 ", "")
        procs.append(subprocess.Popen(["bash", "-c", cmd]))
    if force or not _newer(run, shim_src):
        procs.append(subprocess.Popen(["gcc", "-O2", os.path.join(shim, "mpishim_run.c"), "-o", run, "-lpthread", "-lrt"]))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("reference MPI build failed")
    return {"simple_ts_mpi_resid": exe, "mpishim_run": run}


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
    print(build_reference_mpi(force="--force" in sys.argv))
