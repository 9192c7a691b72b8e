"""TEST INFRASTRUCTURE: ctypes binding of the CPU oracle (oracle/sts_oracle.cpp).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module, always as the checker of the GB300 library, never as a substitute for it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libsts_oracle.so")
EXE = os.path.join(HERE, "_build", "sts_oracle")
REF_FIXED = os.path.join(HERE, "_ref", "simple_ts_fixed")
REF_RESID = os.path.join(HERE, "_ref", "simple_ts_resid")

_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            from build_oracle import build_oracle  # noqa: F401  (oracle/ on sys.path)
            build_oracle()
        lib = C.CDLL(LIB)
        P = C.c_void_p
        lib.ora_open.argtypes = [C.c_char_p, C.c_int, C.c_int]
        lib.ora_open.restype = P
        lib.ora_step.argtypes = [P, C.c_int]
        lib.ora_finish.argtypes = [P]
        lib.ora_close.argtypes = [P]
        lib.ora_dims.argtypes = [P, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        lib.ora_get.argtypes = [P, C.c_char_p, C.POINTER(C.c_double)]
        lib.ora_get_mask.argtypes = [P, C.POINTER(C.c_uint)]
        lib.ora_get_class.argtypes = [P, C.POINTER(C.c_ubyte)]
        lib.ora_sweeps.argtypes = [P, C.POINTER(C.c_uint), C.c_int]
        lib.ora_stats.argtypes = [P, C.POINTER(C.c_double)]
        lib.ora_set_warm_start.argtypes = [P, C.c_int]
        lib.ora_set_guess.argtypes = [P, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        lib.ora_conservation.argtypes = [P, C.POINTER(C.c_double)]
        _lib = lib
    return _lib


class Oracle:
    def __init__(self, case_dir, fixed_sweeps=True, write_files=False, warm_start=0):
        lib = load()
        self._h = lib.ora_open(case_dir.encode(), int(fixed_sweeps), int(write_files))
        if not self._h:
            raise RuntimeError(f"oracle could not open {case_dir}")
        if warm_start:
            lib.ora_set_warm_start(self._h, int(warm_start))
        nx, ny = C.c_int(), C.c_int()
        lib.ora_dims(self._h, C.byref(nx), C.byref(ny))
        self.Nx, self.Ny = nx.value, ny.value

    def step(self, n=1):
        return load().ora_step(self._h, int(n))

    def set_guess(self, p, T):
        """The next step's p-T sweeps start from these fields (Nx*Ny each) on the solved cells."""
        pa = np.ascontiguousarray(p, dtype=np.float64).ravel()
        ta = np.ascontiguousarray(T, dtype=np.float64).ravel()
        assert pa.size == ta.size == self.Nx * self.Ny
        self._keep = (pa, ta)
        load().ora_set_guess(self._h, pa.ctypes.data_as(C.POINTER(C.c_double)), ta.ctypes.data_as(C.POINTER(C.c_double)))

    def field(self, name):
        n = self.Nx if name in ("hx", "x_v") else self.Ny if name in ("hy", "y_v") else self.Nx * self.Ny
        out = np.empty(n)
        if load().ora_get(self._h, name.encode(), out.ctypes.data_as(C.POINTER(C.c_double))) != 0:
            raise KeyError(name)
        return out if n != self.Nx * self.Ny else out.reshape(self.Ny, self.Nx)

    def mask(self):
        out = np.empty(self.Nx * self.Ny, dtype=np.uint32)
        load().ora_get_mask(self._h, out.ctypes.data_as(C.POINTER(C.c_uint)))
        return out.reshape(self.Ny, self.Nx)

    def classes(self):
        out = np.empty(self.Nx * self.Ny, dtype=np.uint8)
        load().ora_get_class(self._h, out.ctypes.data_as(C.POINTER(C.c_ubyte)))
        return out.reshape(self.Ny, self.Nx)

    def sweeps(self, cap=1 << 16):
        out = np.zeros(cap, dtype=np.uint32)
        n = load().ora_sweeps(self._h, out.ctypes.data_as(C.POINTER(C.c_uint)), cap)
        return out[:n]

    def stats(self):
        out = np.zeros(9)
        load().ora_stats(self._h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def conservation(self):
        """[mass, x momentum, y momentum, internal energy, kinetic energy] sums of the current
        state over the fluid cells, in the GB300 library's fixed summation order."""
        out = np.zeros(5)
        load().ora_conservation(self._h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def finish(self):
        load().ora_finish(self._h)

    def close(self):
        if self._h:
            load().ora_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pt_sweeps(Nx, Ny, periodic, given_xb, given_xe, Nx_o0, Nx_o1, ht, gamma1, cls, hx, hy, fields, p, T,
              max_sweeps, fixed, tol_p, tol_T):
    """The sweep loop of the oracle on host arrays; fields: dict of the sweep inputs (Nx*Ny each).
    Returns (p, T, sweeps, res_p, res_T)."""
    lib = load()
    dp = C.POINTER(C.c_double)
    names = ["Fx", "Fy", "DTx", "DTy", "u", "v", "rho", "ScT1", "apx", "apy", "bpx", "bpy", "p_pr", "T_pr",
             "Tw_u", "Tw_v"]
    lib.ora_pt_sweeps.argtypes = ([C.c_int] * 7 + [C.c_double] * 2 + [C.POINTER(C.c_ubyte)] + [dp] * 2 +
                                  [dp] * len(names) + [dp, dp, C.c_int, C.c_int, C.c_double, C.c_double,
                                                       C.POINTER(C.c_int), dp, dp])
    arrs = [np.ascontiguousarray(fields[n], dtype=np.float64).reshape(-1) for n in names]
    p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1).copy()
    T = np.ascontiguousarray(T, dtype=np.float64).reshape(-1).copy()
    cls = np.ascontiguousarray(cls, dtype=np.uint8).reshape(-1)
    hx = np.ascontiguousarray(hx, dtype=np.float64)
    hy = np.ascontiguousarray(hy, dtype=np.float64)
    n, rp, rT = C.c_int(), C.c_double(), C.c_double()
    lib.ora_pt_sweeps(Nx, Ny, int(periodic), int(given_xb), int(given_xe), Nx_o0, Nx_o1, ht, gamma1,
                      cls.ctypes.data_as(C.POINTER(C.c_ubyte)), hx.ctypes.data_as(dp), hy.ctypes.data_as(dp),
                      *[a.ctypes.data_as(dp) for a in arrs], p.ctypes.data_as(dp), T.ctypes.data_as(dp),
                      int(max_sweeps), int(fixed), float(tol_p), float(tol_T), C.byref(n), C.byref(rp), C.byref(rT))
    return p.reshape(Ny, Nx), T.reshape(Ny, Nx), n.value, rp.value, rT.value


def run_cli(case_dir, fixed_sweeps=True):
    args = [EXE, case_dir] + ([] if fixed_sweeps else ["--residual"])
    return subprocess.run(args, capture_output=True, text=True, check=True)


def run_reference(case_dir, fixed_sweeps=True):
    exe = REF_FIXED if fixed_sweeps else REF_RESID
    return subprocess.run([exe], cwd=case_dir, capture_output=True, text=True, check=True)
