"""Python binding of libsts_gb300.so (ctypes over the C ABI in include/sts_gb300.h).

The library is the product; this module only loads it and converts arrays.  It
fails loudly when the library has not been built: there is no Python or CPU
fallback for the time step.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsts_gb300.so")
EXE_PATH = os.path.join(HERE, "_build", "simple_ts_gb300")

STS_OK = 0
STS_ERR_ARG = -1
STS_ERR_INPUT = -2
STS_ERR_CUDA = -3
STS_ERR_NONFINITE = -4
STS_ERR_TIMEOUT = -5

# every symbol include/sts_gb300.h declares
EXPORTS = [
    "sts_default_options", "sts_open_case", "sts_step", "sts_get_field", "sts_set_field", "sts_dims",
    "sts_stats", "sts_sweep_history", "sts_write_outputs", "sts_run_case", "sts_sync", "sts_destroy",
    "sts_last_error", "sts_inspect_case", "sts_step_timed", "sts_profile_steps", "sts_pt_sweeps",
    "sts_pt_sweeps_noalloc", "sts_check_division", "sts_fp64_rates", "sts_open_batch", "sts_batch_step", "sts_batch_step_timed",
    "sts_batch_case", "sts_batch_destroy", "sts_check_double_float", "sts_write_outputs_async",
    "sts_wait_outputs", "sts_autotune_result", "sts_set_state", "sts_get_state", "sts_batch_autotune_result",
    "sts_step_exchange", "sts_warm_net_gate",
]

KERNELS = ["step_begin", "assemble", "sweep_loop", "correct", "face_rho", "boundary", "flux_diff", "step_end"]

# precision modes of sts_options.precision
EXACT, FAST_FP64, MIXED, MIXED_DF = 0, 1, 2, 3

FIELDS = ["u", "v", "p", "T", "rho", "sqrt_T", "rho_u", "rho_v", "Fx", "Fy", "D_ux", "D_uy", "D_vx", "D_vy",
          "DTx", "DTy", "Gamma_xf", "Gamma_yf", "ScT1", "apx", "apy", "bpx", "bpy", "u_pseudo", "v_pseudo",
          "d_p_c_12", "d_p_c_34", "Tw_u", "Tw_v"]


class Options(C.Structure):
    _fields_ = [("fixed_sweeps", C.c_int), ("use_graph", C.c_int), ("device", C.c_int), ("write_files", C.c_int),
                ("precision", C.c_int), ("warm_start", C.c_int), ("async_save", C.c_int),
                ("autotune", C.c_int)]


class StsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sts error {code}: {msg}")
        self.code = code


_lib: Optional[C.CDLL] = None


def load(path: str = LIB_PATH) -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: build it with simple-ts_gb300/build.py (no fallback exists)")
    lib = C.CDLL(path)
    P = C.c_void_p
    dp = C.POINTER(C.c_double)
    lib.sts_default_options.argtypes = [C.POINTER(Options)]
    lib.sts_default_options.restype = None
    lib.sts_open_case.argtypes = [C.c_char_p, C.POINTER(Options), C.POINTER(P)]
    lib.sts_step.argtypes = [P, C.c_int, C.POINTER(C.c_int)]
    lib.sts_step_timed.argtypes = [P, C.c_int, C.POINTER(C.c_int), dp]
    lib.sts_profile_steps.argtypes = [P, C.c_int, dp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.sts_get_field.argtypes = [P, C.c_char_p, dp]
    lib.sts_set_field.argtypes = [P, C.c_char_p, dp]
    lib.sts_dims.argtypes = [P, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.sts_stats.argtypes = [P, dp]
    lib.sts_sweep_history.argtypes = [P, C.POINTER(C.c_uint), C.c_int, C.POINTER(C.c_int)]
    lib.sts_write_outputs.argtypes = [P]
    lib.sts_write_outputs_async.argtypes = [P]
    lib.sts_wait_outputs.argtypes = [P]
    ip = C.POINTER(C.c_int)
    lib.sts_autotune_result.argtypes = [P, ip, ip, ip, ip]
    lib.sts_set_state.argtypes = [P, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.sts_get_state.argtypes = [P, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.sts_step_exchange.argtypes = [P, C.c_int] + [C.c_void_p] * 8 + [C.POINTER(C.c_int)]
    lib.sts_run_case.argtypes = [C.c_char_p, C.POINTER(Options)]
    lib.sts_sync.argtypes = [P]
    lib.sts_destroy.argtypes = [P]
    lib.sts_destroy.restype = None
    lib.sts_last_error.argtypes = []
    lib.sts_last_error.restype = C.c_char_p
    lib.sts_inspect_case.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_uint),
                                     C.POINTER(C.c_ubyte), dp, dp, dp, dp]
    _lib = lib
    return lib


def _check(code: int):
    if code != STS_OK:
        raise StsError(code, load().sts_last_error().decode())


def options(fixed_sweeps=True, use_graph=True, device=0, write_files=False, precision=EXACT,
            warm_start=0, async_save=True, autotune=True) -> Options:
    o = Options()
    load().sts_default_options(C.byref(o))
    o.fixed_sweeps = int(fixed_sweeps)
    o.use_graph = int(use_graph)
    o.device = int(device)
    o.write_files = int(write_files)
    o.precision = int(precision)
    o.warm_start = int(warm_start)
    o.async_save = int(async_save)
    o.autotune = int(autotune)
    return o


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Solver:
    """One case on one GPU: the reference's solve loop behind the C ABI."""

    def __init__(self, case_dir: str, fixed_sweeps=True, use_graph=True, device=0, precision=EXACT, warm_start=0,
                 autotune=True, _handle=None):
        lib = load()
        self._owned = _handle is None
        if _handle is None:
            self._h = C.c_void_p()
            opt = options(fixed_sweeps, use_graph, device, False, precision, warm_start, autotune=autotune)
            _check(lib.sts_open_case(case_dir.encode(), C.byref(opt), C.byref(self._h)))
        else:
            self._h = _handle
        nx, ny = C.c_int(), C.c_int()
        _check(lib.sts_dims(self._h, C.byref(nx), C.byref(ny)))
        self.Nx, self.Ny = nx.value, ny.value

    def step(self, n: int = 1, allow_nonfinite: bool = False) -> int:
        done = C.c_int()
        r = load().sts_step(self._h, int(n), C.byref(done))
        if r == STS_ERR_NONFINITE and allow_nonfinite:
            return done.value
        _check(r)
        return done.value

    def step_timed(self, n: int):
        """(steps taken, device milliseconds) measured with CUDA events on the library's stream."""
        done, ms = C.c_int(), C.c_double()
        _check(load().sts_step_timed(self._h, int(n), C.byref(done), C.byref(ms)))
        return done.value, ms.value

    def profile(self, n: int):
        """Per-kernel device time (ms) and launch counts over n real steps."""
        ms = np.zeros(len(KERNELS))
        cnt = np.zeros(len(KERNELS), dtype=np.int32)
        done = C.c_int()
        _check(load().sts_profile_steps(self._h, int(n), _dptr(ms), cnt.ctypes.data_as(C.POINTER(C.c_int)),
                                        C.byref(done)))
        return done.value, dict(zip(KERNELS, ms)), dict(zip(KERNELS, cnt.tolist()))

    def set_field_ptr(self, name: str, host_ptr: int):
        """Upload from a raw host pointer (e.g. a pinned buffer) of Nx*Ny doubles."""
        _check(load().sts_set_field(self._h, name.encode(), C.cast(C.c_void_p(host_ptr), C.POINTER(C.c_double))))

    def get_field_ptr(self, name: str, host_ptr: int):
        _check(load().sts_get_field(self._h, name.encode(), C.cast(C.c_void_p(host_ptr), C.POINTER(C.c_double))))

    def field(self, name: str) -> np.ndarray:
        n = self.Nx if name in ("hx", "x_v") else self.Ny if name in ("hy", "y_v") else self.Nx * self.Ny
        out = np.empty(n, dtype=np.float64)
        _check(load().sts_get_field(self._h, name.encode(), _dptr(out)))
        return out if n != self.Nx * self.Ny else out.reshape(self.Ny, self.Nx)

    def set_field(self, name: str, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
        _check(load().sts_set_field(self._h, name.encode(), _dptr(a)))

    def stats(self) -> np.ndarray:
        out = np.zeros(9)
        _check(load().sts_stats(self._h, _dptr(out)))
        return out

    def set_sweep_blocking(self, k: int):
        """FP32 correction sweeps per tile load: 1, 2, or 0 for the autotuner's choice."""
        _check(load().sts_set_sweep_blocking(self._h, int(k)))

    def sweep_blocking(self) -> int:
        k = C.c_int()
        _check(load().sts_get_sweep_blocking(self._h, C.byref(k)))
        return k.value

    def warm_net_train(self, iters: int, lr: float = 1e-3) -> float:
        """warm_start 5: Adam steps of the network on the stored training pairs; the last loss."""
        lib = load()
        lib.sts_warm_net_train.argtypes = [C.c_void_p, C.c_int, C.c_float, C.POINTER(C.c_float)]
        loss = C.c_float()
        _check(lib.sts_warm_net_train(self._h, int(iters), float(lr), C.byref(loss)))
        return loss.value

    def warm_net_eval(self):
        """(network loss, zero-correction loss) over every stored training pair."""
        lib = load()
        lib.sts_warm_net_eval.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        a, b = C.c_float(), C.c_float()
        _check(lib.sts_warm_net_eval(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def warm_net_enable(self, on: bool = True):
        _check(load().sts_warm_net_enable(self._h, int(on)))

    def warm_net_info(self) -> dict:
        lib = load()
        lib.sts_warm_net_info.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                          C.POINTER(C.c_longlong)]
        v = [C.c_int(), C.c_int(), C.c_int()]
        n = C.c_longlong()
        _check(lib.sts_warm_net_info(self._h, *[C.byref(x) for x in v], C.byref(n)))
        return {"pairs": v[0].value, "window": (v[1].value, v[2].value), "params": n.value}

    def warm_net_gate(self) -> dict:
        """Steps whose window took the network's correction of p and of T (sts_warm_net_gate)."""
        lib = load()
        lib.sts_warm_net_gate.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        a, b = C.c_int(), C.c_int()
        _check(lib.sts_warm_net_gate(self._h, C.byref(a), C.byref(b)))
        return {"p": a.value, "T": b.value}

    def warm_net_params(self, new=None) -> np.ndarray:
        """The network's FP32 parameters; with `new`, sets them (returning the old ones)."""
        lib = load()
        lib.sts_warm_net_params.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        out = np.zeros(self.warm_net_info()["params"], np.float32)
        src = None
        if new is not None:
            src = np.ascontiguousarray(new, np.float32)
            assert src.size == out.size
        _check(lib.sts_warm_net_params(self._h, out.ctypes.data, None if src is None else src.ctypes.data))
        return out

    def conservation(self) -> np.ndarray:
        """[mass, x momentum, y momentum, internal energy, kinetic energy] sums of the current state
        over the fluid cells (FP64, fixed order, on the device)."""
        out = np.zeros(5)
        _check(load().sts_conservation(self._h, _dptr(out)))
        return out

    def sweep_history(self, cap: int = 4096) -> np.ndarray:
        out = np.zeros(cap, dtype=np.uint32)
        n = C.c_int()
        _check(load().sts_sweep_history(self._h, out.ctypes.data_as(C.POINTER(C.c_uint)), cap, C.byref(n)))
        return out[: n.value]

    def write_outputs(self):
        """The reference's dumps of the current state, on disk when this returns."""
        _check(load().sts_write_outputs(self._h))

    def write_outputs_async(self):
        """The same dumps, written from a host thread while later steps run; complete after
        wait_outputs(), write_outputs() or close()."""
        _check(load().sts_write_outputs_async(self._h))

    def wait_outputs(self):
        _check(load().sts_wait_outputs(self._h))

    def set_state_ptr(self, u, v, p, T):
        """u, v, p, T from raw host pointers (Nx*Ny doubles each) in one call."""
        _check(load().sts_set_state(self._h, u, v, p, T))

    def get_state_ptr(self, u, v, p, T):
        """u, v, p, T to raw host pointers (Nx*Ny doubles each) in one call."""
        _check(load().sts_get_state(self._h, u, v, p, T))

    def step_exchange_ptr(self, n: int, ins, outs) -> int:
        """u, v, p, T in from raw host pointers, n steps, u, v, p, T out to raw host pointers, with
        one synchronisation (sts_step_exchange); returns the steps taken."""
        done = C.c_int()
        _check(load().sts_step_exchange(self._h, int(n), *ins, *outs, C.byref(done)))
        return done.value

    def autotune_result(self) -> dict:
        """Launch shapes in use: tuning steps still to come, sweep-loop CTAs per SM, assembly block."""
        v = [C.c_int() for _ in range(4)]
        _check(load().sts_autotune_result(self._h, *[C.byref(x) for x in v]))
        return {"steps_left": v[0].value, "ctas_per_sm": v[1].value, "asm_block": (v[2].value, v[3].value)}

    def sync(self):
        _check(load().sts_sync(self._h))

    def close(self):
        if self._h:
            if self._owned:
                load().sts_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_case(case_dir: str, fixed_sweeps=True, use_graph=True, device=0, write_files=True, precision=EXACT,
             async_save=True):
    """The drop-in run: same effect as the reference binary in case_dir."""
    opt = options(fixed_sweeps, use_graph, device, write_files, precision, async_save=async_save)
    _check(load().sts_run_case(case_dir.encode(), C.byref(opt)))


def inspect_case(case_dir: str) -> dict:
    """Host-only set-up results (no GPU needed): mask, per-cell classes and mesh."""
    lib = load()
    nx, ny = C.c_int(), C.c_int()
    _check(lib.sts_inspect_case(case_dir.encode(), C.byref(nx), C.byref(ny), None, None, None, None, None, None))
    Nx, Ny = nx.value, ny.value
    vol = np.empty(Nx * Ny, dtype=np.uint32)
    cls = np.empty(Nx * Ny, dtype=np.uint8)
    hx, hy, xv, yv = np.empty(Nx), np.empty(Ny), np.empty(Nx), np.empty(Ny)
    _check(lib.sts_inspect_case(case_dir.encode(), C.byref(nx), C.byref(ny),
                                vol.ctypes.data_as(C.POINTER(C.c_uint)), cls.ctypes.data_as(C.POINTER(C.c_ubyte)),
                                _dptr(hx), _dptr(hy), _dptr(xv), _dptr(yv)))
    return dict(Nx=Nx, Ny=Ny, vol=vol.reshape(Ny, Nx), cls=cls.reshape(Ny, Nx), hx=hx, hy=hy, x_v=xv, y_v=yv)


class SweepFields(C.Structure):
    """sts_sweep_fields: device pointers (ints) of the sweep inputs."""
    _fields_ = [("Nx", C.c_int), ("Ny", C.c_int), ("periodic", C.c_int), ("given_u_xb", C.c_int),
                ("given_u_xe", C.c_int), ("Nx_o0", C.c_int), ("Nx_o1", C.c_int), ("ht", C.c_double),
                ("gamma1", C.c_double)] + [(n, C.c_void_p) for n in (
                    "cls", "hx", "hy", "Fx", "Fy", "DTx", "DTy", "u", "v", "rho", "ScT1", "apx", "apy", "bpx", "bpy",
                    "p_pr", "T_pr", "Tw_u", "Tw_v", "p", "T")]


SWEEP_INPUTS = ["Fx", "Fy", "DTx", "DTy", "u", "v", "rho", "ScT1", "apx", "apy", "bpx", "bpy", "p_pr", "T_pr",
                "Tw_u", "Tw_v"]


def pt_sweeps(fields: SweepFields, max_sweeps: int, fixed_sweeps: bool, tol_p: float, tol_T: float,
              stream: int = 0):
    """Runs the p-T sweep loop on device arrays; returns (sweeps, res_p, res_T)."""
    lib = load()
    lib.sts_pt_sweeps.argtypes = [C.POINTER(SweepFields), C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p,
                                  C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    n, rp, rT = C.c_int(), C.c_double(), C.c_double()
    _check(lib.sts_pt_sweeps(C.byref(fields), int(max_sweeps), int(fixed_sweeps), float(tol_p), float(tol_T),
                             C.c_void_p(stream), C.byref(n), C.byref(rp), C.byref(rT)))
    return n.value, rp.value, rT.value


def pt_sweeps_noalloc(fields: SweepFields, max_sweeps: int, fixed_sweeps: bool, tol_p: float, tol_T: float,
                      stream: int = 0):
    """sts_pt_sweeps_noalloc: the same loop for callers that must not allocate device memory
    (scratch in the library's fixed device array, meshes up to STS_NOALLOC_MAX_CELLS cells)."""
    lib = load()
    lib.sts_pt_sweeps_noalloc.argtypes = [C.POINTER(SweepFields), C.c_int, C.c_int, C.c_double, C.c_double,
                                          C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                          C.POINTER(C.c_double)]
    n, rp, rT = C.c_int(), C.c_double(), C.c_double()
    _check(lib.sts_pt_sweeps_noalloc(C.byref(fields), int(max_sweeps), int(fixed_sweeps), float(tol_p),
                                     float(tol_T), C.c_void_p(stream), C.byref(n), C.byref(rp), C.byref(rT)))
    return n.value, rp.value, rT.value


def check_division(n: int, seed: int = 1, device: int = 0) -> int:
    """Results (of n pairs) where the library's reciprocal-based division, or its IEEE division
    with zero dividends answered directly, differs from IEEE division in any bit."""
    lib = load()
    lib.sts_check_division.argtypes = [C.c_ulonglong, C.c_ulonglong, C.c_int, C.POINTER(C.c_ulonglong)]
    out = C.c_ulonglong()
    _check(lib.sts_check_division(int(n), int(seed), int(device), C.byref(out)))
    return out.value


def check_barrier_timeout(skip_cta: int, spin_limit: int, rounds: int = 1, device: int = 0) -> int:
    """The grid barrier's bounded wait: STS_OK when all `rounds` barriers completed, STS_ERR_TIMEOUT
    when a wait gave up (skip_cta >= 0 leaves one CTA out of the barrier)."""
    lib = load()
    lib.sts_check_barrier_timeout.argtypes = [C.c_int, C.c_int, C.c_uint, C.c_int]
    r = lib.sts_check_barrier_timeout(int(device), int(skip_cta), int(spin_limit), int(rounds))
    if r not in (STS_OK, STS_ERR_TIMEOUT):
        _check(r)
    return r


def fp64_rates(device: int = 0):
    """Measured FP64 add, multiply and fused multiply-add rates of the device (10^9 op/s)."""
    lib = load()
    lib.sts_fp64_rates.argtypes = [C.c_int, C.POINTER(C.c_double)]
    out = (C.c_double * 3)()
    _check(lib.sts_fp64_rates(int(device), out))
    return {"add": out[0], "mul": out[1], "fma": out[2]}


class Batch:
    """Many independent cases advanced together (one launch per kernel and step for all)."""

    def __init__(self, case_dirs, fixed_sweeps=False, device=0, precision=EXACT, warm_start=0, use_graph=True,
                 autotune=True):
        lib = load()
        lib.sts_open_batch.argtypes = [C.POINTER(C.c_char_p), C.c_int, C.POINTER(Options), C.POINTER(C.c_void_p)]
        lib.sts_batch_step.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int)]
        lib.sts_batch_step_timed.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]
        lib.sts_batch_case.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
        lib.sts_batch_destroy.argtypes = [C.c_void_p]
        ip = C.POINTER(C.c_int)
        lib.sts_batch_autotune_result.argtypes = [C.c_void_p, ip, ip, ip, ip]
        dirs = (C.c_char_p * len(case_dirs))(*[d.encode() for d in case_dirs])
        self._h = C.c_void_p()
        opt = options(fixed_sweeps, use_graph, device, False, precision, warm_start, autotune=autotune)
        _check(lib.sts_open_batch(dirs, len(case_dirs), C.byref(opt), C.byref(self._h)))
        self.cases = []
        for k in range(len(case_dirs)):
            h = C.c_void_p()
            _check(lib.sts_batch_case(self._h, k, C.byref(h)))
            self.cases.append(Solver("", _handle=h))

    def step(self, n: int = 1) -> int:
        done = C.c_int()
        _check(load().sts_batch_step(self._h, int(n), C.byref(done)))
        return done.value

    def autotune_result(self) -> dict:
        """Launch shapes in use: tuning steps still to come, sweep-loop CTAs per SM, assembly block."""
        v = [C.c_int() for _ in range(4)]
        _check(load().sts_batch_autotune_result(self._h, *[C.byref(x) for x in v]))
        return {"steps_left": v[0].value, "ctas_per_sm": v[1].value, "asm_block": (v[2].value, v[3].value)}

    def step_timed(self, n: int):
        done, ms = C.c_int(), C.c_double()
        _check(load().sts_batch_step_timed(self._h, int(n), C.byref(done), C.byref(ms)))
        return done.value, ms.value

    def close(self):
        if self._h:
            for c in self.cases:
                c._h = C.c_void_p()
            load().sts_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def check_double_float(n: int, seed: int = 1, device: int = 0):
    """Largest relative errors of the double-float conversion, add, multiply, divide and sqrt."""
    lib = load()
    lib.sts_check_double_float.argtypes = [C.c_ulonglong, C.c_ulonglong, C.c_int, C.POINTER(C.c_double)]
    out = (C.c_double * 5)()
    _check(lib.sts_check_double_float(int(n), int(seed), int(device), out))
    return dict(zip(["convert", "add", "mul", "div", "sqrt"], list(out)))
