"""Builds libsts_gb300.so and the simple_ts_gb300 drop-in executable for sm_103a.

Everything lands in simple-ts_gb300/_build/ (in-tree, git-ignored).  The FP64
kernels that must match the reference bit for bit are compiled with
--fmad=false; host code uses -ffp-contract=off so that Arm and x86 hosts round
the set-up arithmetic identically.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off"]

UNITS = [
    # (source, extra flags)
    ("sts_exact.cu", ["--fmad=false"]),
    ("sts_fast.cu", []),
    ("sts_learn.cu", ["--fmad=false"]),
    ("sts_net.cu", []),
    ("sts_unet.cu", []),
    ("sts_warmnet.cu", []),
    ("sts_runtime.cu", []),
    ("sts_host.cpp", []),
    ("sts_checkpoint.cpp", []),
]

LIB = os.path.join(BUILD, "libsts_gb300.so")
EXE = os.path.join(BUILD, "simple_ts_gb300")


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(os.path.dirname(HERE), "include", "sts_gb300.h"))
    return hs


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = _headers()
    objs, procs = [], []
    for src, extra in UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmd = [NVCC] + ARCH + COMMON + extra + ["-c", s, "-o", o]
            if src.endswith(".cpp"):
                cmd = [NVCC, "-x", "cu"] + ARCH + COMMON + extra + ["-c", s, "-o", o]
            if verbose:
                print(" ".join(cmd))
            procs.append((src, subprocess.Popen(cmd)))
    for src, p in procs:
        if p.wait() != 0:
            raise RuntimeError(f"compiling {src} failed")
    if force or _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcuda", "-lpthread"]
        subprocess.check_call(cmd)
    main = os.path.join(CSRC, "sts_main.cpp")
    if force or _stale(EXE, [main, LIB]):
        cmd = ["g++", "-O2", "-std=c++17", main, "-o", EXE, "-L" + BUILD, "-lsts_gb300",
               "-Wl,-rpath,$ORIGIN"]
        subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
