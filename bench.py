"""Benchmark of the GB300 SIMPLE-TS time step (one JSON line on rank 0).

Workload: the supersonic channel with a confined square (1200x120 fluid cells,
Mach 2.43, Kn 0.00283, dt 2.5e-4), p-T Jacobi sweeps iterated to the 1e-8 update
residual every step, FP64.  A "step" is one time step of the solver.  Inputs are
synthetic case files generated by sts_cases.py (no dataset is involved).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

With N > 1 (torchrun, one rank per GPU) every rank advances its own copy of the
case: the path shards by independent cases, there is no collective on the data
path, scaling is weak.  The timed region of every rank is bracketed by a barrier
and a device synchronisation; the slowest rank's time is reported.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.join(ROOT, "simple-ts_gb300"), os.path.join(ROOT, "oracle")]

METRIC = "cell-steps/s at fixed residual: learned warm-start vs plain Jacobi; % HBM peak"
UNIT = "cell-steps/s"
WORKLOAD = "channel_ma2.43"
L2_BYTES = 129 * 2 ** 20

# algorithmic bytes per cell and launch of each kernel: arrays the kernel must read once and
# write once for one cell, 8 bytes each, plus the 1-byte class
BYTES_PER_CELL = {
    "sweep_loop": 32,     # per sweep: read p, T of the iterate, write p, T (times sweeps per launch)
    "assemble": 27 * 8 + 1,
    "flux_diff": 21 * 8 + 1,  # with the six static quotient tables
    "correct": 10 * 8 + 1,
    "face_rho": 5 * 8 + 1,
    "step_begin": 10 * 8,
}

# DRAM bytes per launch measured by ncu on the default workload (the 1200x120 channel), FP64 path (dram__bytes_read.sum +
# dram__bytes_write.sum of one launch of the fourteenth time step, cold cache); None where no
# capture was taken
TRAFFIC = {"assemble": 21101056, "sweep_loop": 19600128 + 20480, "flux_diff": 16722432}

# FP64 instructions per cell of the FP64 path's kernels (per cell and sweep for the sweep loop),
# counted by ncu on this workload (smsp__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on
# of one launch divided by its 1203 x 123 cells and, for the sweep loop, by its 8 sweeps).  The
# kernels are bound by the FP64 unit, so their roofline is this work at the device's measured
# FP64 rates (sts_fp64_rates) against the measured launch time.
FP64_OPS = {"assemble": {"add": 94.24, "mul": 104.97, "fma": 29.69},
            "sweep_loop": {"add": 20.64, "mul": 16.55, "fma": 19.22},
            "flux_diff": {"add": 14.28, "mul": 42.42, "fma": 32.74}}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--warm-lead", type=int, default=40,
                    help="untimed steps before the timed ones for warm-started variants (the learned "
                         "predictors fit on the run's own history, which fills in the first 10 steps)")
    ap.add_argument("--variant-set", default="all", choices=["all", "warm"],
                    help="which variants to time: all of them, or only the warm-start comparison "
                         "(plain FP64 against the extrapolated and learned starts) without the "
                         "checkpoint and untuned-shape lines")
    ap.add_argument("--c5-steps", type=int, default=20,
                    help="timed steps per path of the 2048x256 metric-configuration runs (0: skip them)")
    ap.add_argument("--c5-lead", type=int, default=30,
                    help="untimed steps before the timed ones for the warm-started paths of those runs")
    ap.add_argument("--no-network", dest="network", action="store_false",
                    help="skip the network warm start (warm_start 5) runs")
    ap.add_argument("--no-variants", dest="variants", action="store_false",
                    help="skip the FP64-fast and FP32-correction runs of the same workload")
    ap.add_argument("--precision", type=int, default=0, choices=[0, 1, 2, 3],
                    help="precision mode of the --profile-target run")
    ap.add_argument("--warm-start", type=int, default=0, choices=[0, 1, 2, 3, 4],
                    help="warm start of the --profile-target run")
    ap.add_argument("--sweep-blocking", type=int, default=0, choices=[0, 1, 2],
                    help="FP32 correction sweeps per tile load for the --profile-target run (0: autotuner)")
    ap.add_argument("--gemm-target", type=int, nargs=3, default=None, metavar=("M", "N", "K"),
                    help="only run the network's tensor-core GEMM self-check twice on seeded BF16 data of "
                         "this shape (a small target for ncu), then exit")
    ap.add_argument("--profile-target", type=int, default=0,
                    help="only run this many steps kernel by kernel (a small target for ncu), then exit")
    return ap.parse_args()


def profile_target(args):
    """A short, plain run of the workload (launch by launch) for an external profiler."""
    import sts
    import build as stsbuild
    stsbuild.build()
    if args.workload == "batch64":
        dirs = batch_dirs()
        b = sts.Batch(dirs, fixed_sweeps=False, precision=args.precision, use_graph=False, warm_start=args.warm_start)
        b.step(args.profile_target)
        print(f"profile target: batch64, {args.profile_target} steps, {sum(c.Nx * c.Ny for c in b.cases)} cells")
        b.close()
        return
    _, d = make_case(args.workload)
    s = sts.Solver(d, fixed_sweeps=False, use_graph=False, precision=args.precision, warm_start=args.warm_start,
                   autotune=args.sweep_blocking == 0)
    if args.sweep_blocking:
        s.set_sweep_blocking(args.sweep_blocking)
    s.step(args.profile_target)
    s.sync()
    print(f"profile target: {args.workload}, {args.profile_target} steps, sweeps {list(s.sweep_history())}")
    s.close()


def gemm_target(M, N, K):
    """The BF16 tensor-core GEMM (sts_tc_gemm) twice on seeded data: D = A B^T, A [M x K], B [N x K]."""
    import ctypes as C
    import numpy as np
    import sts
    import build as stsbuild
    stsbuild.build()
    lib = sts.load()
    lib.sts_tc_gemm.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                C.c_int]
    rng = np.random.default_rng(0)

    def bf16(x):
        u = x.astype(np.float32).view(np.uint32)
        return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)

    A = bf16(rng.standard_normal((M, K)) * 0.1)
    B = bf16(rng.standard_normal((N, K)) * 0.1)
    D = np.zeros((M, N), np.float32)
    for _ in range(2):
        r = lib.sts_tc_gemm(A.ctypes.data, B.ctypes.data, M, N, K, 0, None, D.ctypes.data, 0)
        if r != 0:
            raise RuntimeError(f"sts_tc_gemm returned {r}")
    print(f"gemm target: {M} x {N} x {K}")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def slowest(x, world, device="cuda"):
    """The largest x over all ranks: a job's time is that of its slowest rank."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, seconds):
    """Whole-job throughput: every rank advanced its own replica by units_per_rank in at most
    `seconds` (weak scaling, no collective on the data path)."""
    return units_per_rank * world / seconds


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d["hbm_gbs"], "measured"
    except Exception:
        return 6800.0, "fallback"


def fp64_roof(dom, kms, kcnt, psweeps, Na, device):
    """The FP64-unit roofline of the dominant kernel: its counted FP64 instructions per launch
    at the device's measured add/multiply/FMA rates, against its measured launch time."""
    import sts
    ops = FP64_OPS.get(dom)
    if not ops or not kcnt.get(dom):
        return None
    rates = sts.fp64_rates(device)
    units = float(Na)
    if dom == "sweep_loop":
        units *= float(sum(int(x) for x in psweeps)) / kcnt[dom]
    launch_s = kms[dom] / 1e3 / kcnt[dom]
    roof_s = sum(ops[k] * units / (rates[k] * 1e9) for k in ops)
    total = sum(ops.values()) * units
    return {"achieved": total / launch_s / 1e9, "peak_at_mix": total / roof_s / 1e9, "unit": "FP64 Gop/s",
            "frac": roof_s / launch_s, "ops_per_cell": ops, "measured_rates_gops": rates,
            "source": "FP64 instruction counts per cell from ncu; rates measured on this GPU by sts_fp64_rates"}


def make_case(workload):
    import sts_cases as sc
    case = sc.config_case(workload, Nt=10 ** 7)
    d = tempfile.mkdtemp(prefix="sts_bench_")
    case.write(d)
    return case, d


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def _replica_worker(case_dir, warm_steps, steps, seconds, start, q):
    """One oracle replica on one host core: set-up and warm-up steps, then (after every replica is
    ready) timed steps -- `steps` of them, or as many as fit in `seconds` when steps is 0."""
    import sys
    sys.path[:0] = [os.path.join(ROOT, "simple-ts_gb300"), os.path.join(ROOT, "oracle")]
    import ora
    o = ora.Oracle(case_dir, fixed_sweeps=False)
    if warm_steps:
        o.step(warm_steps)
    start.wait()
    n, t0 = 0, time.perf_counter()
    while True:
        n += o.step(1)
        dt = time.perf_counter() - t0
        if (steps and n >= steps) or (not steps and ((dt >= seconds and n >= 2) or n >= 10000)):
            break
    q.put((o.Nx * o.Ny, n, dt))


def cpu_replicas(case_dir, procs, warm_steps=0, steps=0, seconds=0.0):
    """The oracle (serial C++ restatement of the reference) on `procs` host cores at once: one
    independent replica of the case per core, started together after their set-up.  Returns the
    host's aggregate cell-steps/s (the sum over replicas) and the per-replica samples.  The pool is
    started with spawn, so it never inherits a CUDA context."""
    import multiprocessing as mpr
    from build_oracle import build_oracle
    build_oracle()
    import queue
    ctx = mpr.get_context("spawn")
    start = ctx.Barrier(procs, timeout=600)
    q = ctx.Queue()
    ps = [ctx.Process(target=_replica_worker, args=(case_dir, warm_steps, steps, seconds, start, q), daemon=True)
          for _ in range(procs)]
    for p in ps:
        p.start()
    res = []
    try:
        for _ in ps:
            res.append(q.get(timeout=900))
    except queue.Empty:
        raise RuntimeError(f"CPU baseline: {len(res)} of {procs} oracle replicas reported")
    finally:
        for p in ps:
            p.join(timeout=5)
            if p.is_alive():
                p.terminate()
    return sum(c * n / dt for c, n, dt in res), res


def cpu_baseline(case_dir, seconds, start_steps=0):
    """The oracle (serial C++ restatement of the reference, bit-identical with the reference binary)
    on this host: one replica of the case per host core, all timed together for a bounded time;
    `value` is the host's aggregate cell-steps/s.  The reference solver is serial without MPI, so
    independent replicas are how it uses every core.  The one-core rate is reported beside it."""
    procs = host_cores()
    agg, res = cpu_replicas(case_dir, procs, warm_steps=start_steps, seconds=seconds)
    one, one_res = cpu_replicas(case_dir, 1, warm_steps=start_steps, seconds=min(seconds, 5.0))
    steps = [n for _, n, _ in res]
    return {"value": agg, "unit": UNIT, "cores": procs, "kind": "port",
            "sample": f"{procs} concurrent replicas of the same case, one per host core, each timed for "
                      f"about {seconds:.0f} s ({min(steps)}-{max(steps)} time steps each) after {start_steps} "
                      "untimed steps; serial oracle, bit-identical with the reference binary",
            "single_core": {"value": one, "cores": 1, "steps": one_res[0][1]}}


def reference_arm(args):
    """The reference's CPU path (the oracle port: the reference tree is not on the GPU host) on
    every host core: one replica of the case per core, W warm-up steps, then K timed steps each;
    the line's value is the host's aggregate cell-steps/s.  Rank 0 only."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    case, d = make_case(args.workload)
    procs = host_cores()
    t0 = time.perf_counter()
    agg, res = cpu_replicas(d, procs, warm_steps=args.warmup, steps=args.steps)
    wall = time.perf_counter() - t0
    cells, n, dt = res[0]
    Nx, Ny = case.Nx, case.Ny
    cfg = config(case, Nx, Ny)
    line = {"impl": "reference", "metric": METRIC, "value": agg, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": max(x[2] / x[1] for x in res) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": cfg,
            "cpu_baseline": {"value": agg, "unit": UNIT, "cores": procs, "kind": "port",
                             "sample": f"{procs} concurrent replicas of the case, one per host core, each "
                                       f"{args.warmup} warm-up + {args.steps} timed time steps; serial oracle "
                                       "(the reference solver is serial without MPI)"},
            "e2e": {"value": agg, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": round(wall, 2)}
    print(json.dumps(line), flush=True)


def config(case, Nx, Ny):
    e = case.entered
    return {"workload": case.name + f" {Nx - 3}x{Ny - 3} fluid cells, square obstacle, slip/jump walls",
            "Nx": Nx, "Ny": Ny, "cells_per_step": Nx * Ny, "mach": 2.43, "Kn": e["Kn"], "dt": e["ht"],
            "residual_tolerance": e["MaxError_p_c"], "method": "plain Jacobi (p-T), FP64 bit-exact with the reference",
            "l2": "flushed before every timed step (256 MiB write); working set 42 MB < L2"}


def timed_steps(s, steps, warmup, flush, barrier, clocks=None):
    """Autotuning steps and warm-up, then `steps` steps each after an L2 flush; device ms from CUDA
    events on the library's stream.  Returns (steps done, total device ms, sweeps of the timed
    steps)."""
    import torch
    # the autotuner's steps (real steps, launched kernel by kernel) come before the warm-up
    pre = max(warmup, 3) + s.autotune_result()["steps_left"]
    for _ in range(pre):
        s.step(1)
    s.sync()
    barrier()
    total_ms, done = 0.0, 0
    ctx = clocks if clocks is not None else _Null()
    with ctx:
        for _ in range(steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            n, ms = s.step_timed(1)
            total_ms += ms
            done += n
    barrier()
    s.steps_before_timing = pre
    return done, total_ms, (s.sweep_history()[-done:] if done else [])


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        pass


def launches_per_step(kcnt, pn):
    """Kernels one step launches (the whole sweep loop is one), from a kernel-by-kernel profile pass."""
    return sum(kcnt.values()) / max(pn, 1)


def partition_cases(cells, world):
    """Shards independent cases over `world` ranks: largest case first, each to the rank with the
    fewest cells so far (ties to the lower rank).  Returns one sorted list of case indices per
    rank; every case is in exactly one list.  Deterministic, so every rank computes the same."""
    load = [0] * world
    parts = [[] for _ in range(world)]
    for k in sorted(range(len(cells)), key=lambda k: (-cells[k], k)):
        r = min(range(world), key=lambda r: (load[r], r))
        parts[r].append(k)
        load[r] += cells[k]
    return [sorted(p) for p in parts]


def batch_dirs(indices=None):
    """Case directories of the 64-case batch (seed 20261204), or of the cases `indices` of it."""
    import sts_cases as sc
    cases = sc.batch_cases(n=64, Nt=10 ** 7)
    root = tempfile.mkdtemp(prefix="sts_batch_")
    dirs = []
    for k, c in enumerate(cases):
        if indices is not None and k not in indices:
            continue
        d = os.path.join(root, f"c{k:02d}")
        os.makedirs(d)
        c.write(d)
        dirs.append(d)
    return dirs


def batch_cells():
    import sts_cases as sc
    return [c.Nx * c.Ny for c in sc.batch_cases(n=64, Nt=10 ** 7)]


def batch_bench(args):
    """The 64-case batch (nx ~ U{200..800}, ny = nx/10, Mach, Kn and square position drawn
    with seed 20261204): all cases advance together, one launch per kernel and step.  With
    N > 1 ranks the cases are sharded over the GPUs (partition_cases; no collective on the data
    path): every rank advances its share as one batch, the job's time is the slowest rank's and
    the value counts every case's cells.  Prints a JSON line of the same shape as the main bench
    (no e2e, no CPU baseline)."""
    import numpy as np
    import torch
    import sts
    import build as stsbuild
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    stsbuild.build()
    all_cells = batch_cells()
    mine = partition_cases(all_cells, world)[rank]
    dirs = batch_dirs(set(mine))
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    out = {}
    base = None
    variants = (("fp64_exact", sts.EXACT, 0), ("fp64_fast", sts.FAST_FP64, 0),
                ("fp32_corrections", sts.MIXED, 0), ("fp32_corrections_warm2", sts.MIXED, 2),
                ("fp32_corrections_df", sts.MIXED_DF, 0), ("fp32_corrections_df_warm2", sts.MIXED_DF, 2),
                ("fp32_corrections_learned", sts.MIXED, 3), ("fp32_corrections_conv", sts.MIXED, 4),
                ("fp32_corrections_df_conv", sts.MIXED_DF, 4))
    if not args.variants:
        variants = variants[:1]
    for name, prec, warm in variants:
        b = sts.Batch(dirs, fixed_sweeps=False, precision=prec, warm_start=warm)
        cells = sum(c.Nx * c.Ny for c in b.cases)
        w = max(args.warmup, 3)
        lead = max(args.warm_lead, w) if warm else w
        lead += b.autotune_result()["steps_left"]  # the autotuner's steps come before the warm-up
        for _ in range(lead):
            b.step(1)
        barrier()
        total, done = 0.0, 0
        with Clocks(local) as clk:
            for _ in range(args.steps):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                n, ms = b.step_timed(1)
                total += ms
                done += n
        barrier()
        total = slowest(total, world)
        fields = {f: np.concatenate([c.field(f).ravel() for c in b.cases]) for f in ("u", "v", "p", "T", "rho")}
        sweeps = np.concatenate([c.sweep_history()[-done:] for c in b.cases])
        r = {"value": sum(all_cells) * done / (total / 1e3), "ms_per_step": total / max(done, 1),
             "sweeps_per_step": float(np.mean(sweeps)), "clocks": clk.summary()}
        r["untimed_steps"] = lead
        r["launch_shapes"] = b.autotune_result()
        if name == "fp64_exact":
            base = {lead + done: fields}
        else:
            n_ref = lead + done
            if n_ref not in base:  # the bit-exact fields after the same number of steps
                rb = sts.Batch(dirs, fixed_sweeps=False, precision=sts.EXACT, autotune=False)
                rb.step(n_ref)
                base[n_ref] = {f: np.concatenate([c.field(f).ravel() for c in rb.cases])
                               for f in ("u", "v", "p", "T", "rho")}
                rb.close()
            ref = base[n_ref]
            r["rel_l2_vs_fp64"] = {f: float(np.linalg.norm(fields[f] - ref[f]) / np.linalg.norm(ref[f]))
                                   for f in fields}
        out[name] = r
        b.close()
    head = out["fp64_exact"]
    line = {"metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": head["ms_per_step"], "higher_is_better": True,
            "scaling": "strong" if world > 1 else "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "batch of 64 channel cases, nx ~ U{200..800}, ny = nx/10, seed 20261204",
                       "cells_per_step": sum(all_cells), "residual_tolerance": 1e-8,
                       "sharding": f"{world} rank(s), cases per rank {[len(p) for p in partition_cases(all_cells, world)]}",
                       "l2": "flushed before every timed step (256 MiB write)"},
            "clocks": head["clocks"], "variants": {k: v for k, v in out.items() if k != "fp64_exact"},
            "sweeps_per_step": head["sweeps_per_step"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def checkpoint_bench(d, local, barrier, every=10, saves=10):
    """Milliseconds per FP64 step with the reference's binary dumps (u, v, p, Temper, vol_inf_fb,
    it_begin.txt, EnteredData.txt) written every `every` steps: not at all, synchronously (the
    reference's order: stepping waits for the files), and from the checkpoint thread
    (sts_write_outputs_async; the wait for the last files is inside the timed region)."""
    import sts
    ms = {}
    for mode in ("no_saves", "sync", "async"):
        s = sts.Solver(d, fixed_sweeps=False, use_graph=True, device=local, precision=sts.EXACT, autotune=False)
        s.step(3)
        if mode != "no_saves":
            s.write_outputs()  # the first save makes the snapshot buffers and the writer thread
        barrier()
        t0 = time.perf_counter()
        for _ in range(saves):
            s.step(every)
            if mode == "sync":
                s.write_outputs()
            elif mode == "async":
                s.write_outputs_async()
        s.wait_outputs()
        s.sync()
        ms[mode] = (time.perf_counter() - t0) * 1e3 / (every * saves)
        s.close()
    cost_sync, cost_async = ms["sync"] - ms["no_saves"], ms["async"] - ms["no_saves"]
    Na = s.Nx * s.Ny
    return {"every_steps": every, "saves": saves, "bytes_per_save": Na * (4 * 8 + 4),
            "ms_per_step": {k: round(v, 5) for k, v in ms.items()},
            "save_cost_hidden": round(1.0 - cost_async / cost_sync, 3) if cost_sync > 0 else None}


def blocking_ab(d, local, steps, flush, barrier, lead):
    """One against two FP32 correction sweeps per tile load (the results are the same bits), on the
    FP32-correction path with double-float FP64 parts from a cold start and with the learned stencil:
    cell-steps/s, sweeps per step and the sweep loop's device time per step (kernel-by-kernel
    profile of further steps).  The autotuner still picks the assembly block and CTAs per SM."""
    import numpy as np
    import sts
    out = {}
    for name, warm in (("fp32df_cold", 0), ("fp32df_learned", 4)):
        row = {}
        for k in (1, 2):
            v = sts.Solver(d, fixed_sweeps=False, device=local, precision=sts.MIXED_DF, warm_start=warm)
            v.set_sweep_blocking(k)
            vd, vms, vsw = timed_steps(v, steps, lead if warm else 3, flush, barrier)
            pn, kms, kcnt = v.profile(max(3, min(steps, 10)))
            row[f"k{k}"] = {"value": v.Nx * v.Ny * vd / (vms / 1e3), "ms_per_step": vms / max(vd, 1),
                            "sweeps_per_step": float(np.mean(vsw)) if len(vsw) else 0.0,
                            "sweep_loop_ms_per_step": kms["sweep_loop"] / max(pn, 1),
                            "blocking_in_use": v.sweep_blocking()}
            v.close()
        row["speedup_k2_over_k1"] = row["k2"]["value"] / row["k1"]["value"]
        out[name] = row
    return out


def network_run(d, local, steps, flush, barrier, lead=60, train_iters=300, lr=3e-4, warmup=10):
    """warm_start 5 on FP32 corrections with double-float FP64 parts: `lead` steps that store the
    network's training pairs (the stencil's start is used unchanged meanwhile), `train_iters` Adam
    steps of the U-Net on the GPU, the correction switched on, `warmup` more steps, then `steps`
    timed steps (device time, L2 flushed before each).  Returns the path's numbers and the training
    losses (network against a zero correction, on the stored pairs)."""
    import numpy as np
    import sts
    v = sts.Solver(d, fixed_sweeps=False, device=local, precision=sts.MIXED_DF, warm_start=5)
    v.step(lead)
    t0 = time.perf_counter()
    v.warm_net_train(train_iters, lr)
    train_s = time.perf_counter() - t0
    loss_net, loss_zero = v.warm_net_eval()
    v.warm_net_enable(True)
    gate0 = v.warm_net_gate()
    vd, vms, vsw = timed_steps(v, steps, warmup, flush, barrier)
    info = v.warm_net_info()
    gate1 = v.warm_net_gate()
    out = {"value": v.Nx * v.Ny * vd / (vms / 1e3), "ms_per_step": vms / max(vd, 1),
           "sweeps_per_step": float(np.mean(vsw)) if len(vsw) else 0.0,
           "untimed_steps": lead + v.steps_before_timing,
           "steps_with_correction": {f: gate1[f] - gate0[f] for f in ("p", "T")},  # of the warm-up and timed steps
           "steps_gated": v.steps_before_timing + vd,
           "training": {
               "pairs": min(info["pairs"], 256), "window": info["window"], "params": info["params"],
               "iters": train_iters, "seconds": round(train_s, 3), "loss_network": loss_net,
               "loss_zero_correction": loss_zero}}
    fields = {f: v.field(f) for f in ("u", "v", "p", "T", "rho")}
    total = lead + v.steps_before_timing + vd
    v.close()
    # the stencil alone (warm_start 4: the same run with the network switched off) over the same
    # steps, for the sweeps the network's correction saves or adds
    ref = sts.Solver(d, fixed_sweeps=False, device=local, precision=sts.MIXED_DF, warm_start=4)
    ref.step(total)
    rsw = ref.sweep_history()[-vd:] if vd else []
    ref.close()
    out["stencil_sweeps_same_steps"] = float(np.mean(rsw)) if len(rsw) else 0.0
    return out, fields


# The metric's own configuration: the 2048x256 channel with the square at four Mach numbers
# (Kn 0.003, dt 1.25e-4, tolerance 1e-8); each path from the same initial state
C5_MACHS = (0.1, 0.5, 1.0, 2.43)


def metric_config_bench(args, local, flush, barrier):
    """Plain GPU Jacobi (FP64 bit-exact, cold start) against the warm starts on the 2048x256
    channel at each Mach number: FP32 corrections with double-float FP64 parts from a cold start,
    from quadratic extrapolation and from the learned convolutional predictor, and quadratic
    extrapolation and the learned predictor on the FP64 path.  Per path: cell-steps/s (device time, L2 flushed before every
    timed step), sweeps per step and the largest per-field relative L2 distance from the plain
    path after the same steps; per Mach: the learned start against plain Jacobi and against the
    same precision without it."""
    import numpy as np
    import sts
    import sts_cases as sc
    EX, DF = sts.EXACT, sts.MIXED_DF
    paths = (("plain_fp64", EX, 0), ("fp64_quadratic", EX, 2), ("fp64_learned", EX, 4), ("fp32df_cold", DF, 0),
             ("fp32df_quadratic", DF, 2), ("fp32df_learned", DF, 4))
    out = {}
    for mach in C5_MACHS:
        case = sc.config_case(f"channel_2048_ma{mach}", Nt=10 ** 7)
        d = tempfile.mkdtemp(prefix="sts_c5_")
        case.write(d)
        base = {}

        def base_at(n):
            if n not in base:
                ref = sts.Solver(d, fixed_sweeps=False, device=local, precision=EX, autotune=False)
                ref.step(n)
                base[n] = {f: ref.field(f) for f in ("u", "v", "p", "T", "rho")}
                ref.close()
            return base[n]

        row = {}
        for name, prec, warm in paths:
            v = sts.Solver(d, fixed_sweeps=False, device=local, precision=prec, warm_start=warm)
            lead = max(args.c5_lead, 3) if warm else max(args.warmup, 3)
            vd, vms, vsw = timed_steps(v, args.c5_steps, lead, flush, barrier)
            ref = base_at(v.steps_before_timing + vd)
            err = max(float(np.linalg.norm(v.field(f) - ref[f]) / np.linalg.norm(ref[f])) for f in ref)
            row[name] = {"value": v.Nx * v.Ny * vd / (vms / 1e3), "ms_per_step": vms / max(vd, 1),
                         "sweeps_per_step": float(np.mean(vsw)) if len(vsw) else 0.0,
                         "max_rel_l2_vs_plain": err, "untimed_steps": v.steps_before_timing}
            cells = v.Nx * v.Ny
            v.close()
        if args.network:
            nr, nf = network_run(d, local, args.c5_steps, flush, barrier, lead=args.c5_lead + 30)
            ref = base_at(nr["untimed_steps"] + args.c5_steps)
            nr["max_rel_l2_vs_plain"] = max(float(np.linalg.norm(nf[f] - ref[f]) / np.linalg.norm(ref[f])) for f in ref)
            row["fp32df_network"] = nr
        plain, learned = row["plain_fp64"], row["fp32df_learned"]

        def gain(a, b):
            return {"speedup": row[a]["value"] / row[b]["value"],
                    "sweep_ratio": row[b]["sweeps_per_step"] / max(row[a]["sweeps_per_step"], 1e-30)}
        out[f"ma{mach}"] = {"cells": cells, "paths": row,
                            "learned_vs_plain": gain("fp32df_learned", "plain_fp64"),
                            "learned_vs_same_precision_cold": gain("fp32df_learned", "fp32df_cold"),
                            "learned_vs_quadratic": gain("fp32df_learned", "fp32df_quadratic"),
                            "fp64_learned_vs_plain": gain("fp64_learned", "plain_fp64"),
                            "fp64_learned_vs_fp64_quadratic": gain("fp64_learned", "fp64_quadratic")}
        if "fp32df_network" in row:
            out[f"ma{mach}"]["network_vs_stencil"] = gain("fp32df_network", "fp32df_learned")
            out[f"ma{mach}"]["network_vs_stencil"]["sweep_ratio_same_steps"] = (
                row["fp32df_network"]["stencil_sweeps_same_steps"] / max(row["fp32df_network"]["sweeps_per_step"], 1e-30))
    return {"workload": "channel 2048x256 with the square, Kn 0.003, dt 1.25e-4, tolerance 1e-8",
            "timed_steps": args.c5_steps, "untimed_steps_warm": args.c5_lead, "by_mach": out}


def warm_summary(plain_value, plain_sweeps, variants):
    """The comparison the metric names: warm-started FP32-correction paths against plain GPU
    Jacobi (the FP64 bit-exact path, cold start), at the same per-step residual tolerance --
    the learned predictor (warm_start 3 or 4, the better of them) and the fastest warm start."""
    warm = {k: v for k, v in variants.items() if v.get("warm_start", 0) and v.get("precision_mode", 0) >= 2}
    if not warm or not len(plain_sweeps):
        return None
    ps = float(sum(plain_sweeps) / len(plain_sweeps))

    def entry(name):
        v = warm[name]
        return {"path": name, "value": v["value"], "sweeps_per_step": v["sweeps_per_step"],
                "speedup": v["value"] / plain_value, "sweep_ratio": ps / max(v["sweeps_per_step"], 1e-30)}

    out = {"plain_gpu_jacobi": {"path": "FP64 bit-exact, cold start", "value": plain_value, "sweeps_per_step": ps}}
    learned = [k for k in warm if warm[k]["warm_start"] in (3, 4, 5)]
    if learned:
        out["learned"] = entry(max(learned, key=lambda k: warm[k]["value"]))
    out["fastest"] = entry(max(warm, key=lambda k: warm[k]["value"]))
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    if args.gemm_target:
        return gemm_target(*args.gemm_target)
    if args.profile_target:
        return profile_target(args)
    if args.workload == "batch64":
        return batch_bench(args)
    rank, world, local = dist_env()
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import sts
    import build as stsbuild
    stsbuild.build()
    case, d = make_case(args.workload)
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # headline: the FP64 path, bit-exact with the reference
    s = sts.Solver(d, fixed_sweeps=False, use_graph=True, device=local, precision=sts.EXACT)
    Nx, Ny = s.Nx, s.Ny
    Na = Nx * Ny
    with Clocks(local) as clk:
        done, total_ms, sweeps = timed_steps(s, args.steps, args.warmup, flush, barrier)
    launch_shapes = s.autotune_result()
    total_ms = slowest(total_ms, world)
    value = job_rate(Na * done, world, total_ms / 1e3)

    # e2e through the C ABI with host buffers: per step the state u, v, p, T goes host->device
    # from pinned memory, one step runs, and the new state comes back device->host into the same
    # buffers, in one call (sts_step_exchange: the set-state, step and get-state calls' work with
    # one synchronisation)
    pins = {f: torch.empty(Na, dtype=torch.float64).pin_memory() for f in ("u", "v", "p", "T")}
    ptrs = [pins[f].data_ptr() for f in ("u", "v", "p", "T")]
    s.get_state_ptr(*ptrs)
    for _ in range(3):  # untimed: the exchange's one-step graph is built at its first call
        s.step_exchange_ptr(1, ptrs, ptrs)
    barrier()
    e2e_steps = max(1, min(args.steps, 20))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.step_exchange_ptr(1, ptrs, ptrs)
    barrier()
    e2e_s = slowest(time.perf_counter() - t0, world)
    # the same exchange as three calls (set state, one step, get state: three synchronisations)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.set_state_ptr(*ptrs)
        s.step(1)
        s.get_state_ptr(*ptrs)
    barrier()
    three_s = slowest(time.perf_counter() - t0, world)
    e2e = {"value": job_rate(Na * e2e_steps, world, e2e_s), "unit": UNIT, "h2d_bytes_per_step": 4 * Na * 8,
           "d2h_bytes_per_step": 4 * Na * 8, "call": "sts_step_exchange",
           "three_calls_value": job_rate(Na * e2e_steps, world, three_s)}

    # per-kernel device time over a few more real steps (the roofline's dominant kernel)
    pn, kms, kcnt = s.profile(max(3, min(args.steps, 10)))
    psweeps = s.sweep_history()[-pn:] if pn else []
    launches = int(round(launches_per_step(kcnt, pn) * done))
    dom = max(kms, key=lambda k: kms[k])
    peak, peak_kind = peaks()
    avg_s = kms[dom] / 1e3 / max(kcnt[dom], 1)
    bpc = BYTES_PER_CELL.get(dom, 0)
    if dom == "sweep_loop":  # bytes per launch: per-sweep bytes times the sweeps one launch took
        bpc *= float(sum(int(x) for x in psweeps)) / max(kcnt[dom], 1)
    achieved = bpc * Na / avg_s / 1e9 if bpc else None
    roof = {"bound": "hbm", "kernel": "k_" + dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "traffic": TRAFFIC.get(dom) if args.workload == WORKLOAD else None,
            "peak_source": peak_kind, "bytes_per_cell": bpc, "avg_launch_us": avg_s * 1e6,
            "kernel_share": {k: round(v / max(sum(kms.values()), 1e-30), 4) for k, v in kms.items()},
            "fp64_pipe": fp64_roof(dom, kms, kcnt, psweeps, Na, local)}
    s.close()

    # the same workload in the faster precision modes, from the same initial state, with the
    # per-field relative L2 distance from the FP64 path (bit-exact with the reference) after
    # the same number of steps
    variants = {}
    if args.variants:
        w = max(args.warmup, 3)
        lead_w = max(args.warm_lead, w)
        base = {}

        def base_at(n):
            """The bit-exact path's fields after n steps (launch shapes do not change them)."""
            if n not in base:
                ref = sts.Solver(d, fixed_sweeps=False, use_graph=True, device=local, precision=sts.EXACT,
                                 autotune=False)
                ref.step(n)
                base[n] = {f: ref.field(f) for f in ("u", "v", "p", "T", "rho")}
                ref.close()
            return base[n]

        chosen = (("fp64_fast", sts.FAST_FP64, 0), ("fp32_corrections", sts.MIXED, 0),
                  ("fp32_corrections_df", sts.MIXED_DF, 0), ("fp32_corrections_df_warm2", sts.MIXED_DF, 2),
                  ("fp64_exact_warm2", sts.EXACT, 2), ("fp32_corrections_warm2", sts.MIXED, 2),
                  ("fp32_corrections_learned", sts.MIXED, 3), ("fp64_exact_conv", sts.EXACT, 4),
                  ("fp32_corrections_conv", sts.MIXED, 4), ("fp32_corrections_df_conv", sts.MIXED_DF, 4))
        if args.variant_set == "warm":
            chosen = tuple(x for x in chosen if x[2] in (2, 4))
        for name, prec, warm in chosen:
            v = sts.Solver(d, fixed_sweeps=False, use_graph=True, device=local, precision=prec, warm_start=warm)
            lead = lead_w if warm else w
            vd, vms, vsw = timed_steps(v, args.steps, lead, flush, barrier)
            ref_f = base_at(v.steps_before_timing + vd)
            err = {f: float(np.linalg.norm(v.field(f) - ref_f[f]) / np.linalg.norm(ref_f[f])) for f in ref_f}
            vpn, vkms, vkcnt = v.profile(max(3, min(args.steps, 10)))
            variants[name] = {
                "precision_mode": prec, "warm_start": warm, "untimed_steps": v.steps_before_timing,
                "value": Na * vd * world / (vms / 1e3),
                "ms_per_step": vms / max(vd, 1),
                "speedup_vs_fp64": (Na * vd / (vms / 1e3)) / (Na * done / (total_ms / 1e3)) if done else None,
                "rel_l2_vs_fp64": err,
                "sweeps_per_step": float(np.mean(vsw)) if len(vsw) else 0.0,
                "gpu_launches": int(round(launches_per_step(vkcnt, vpn) * vd)),
                "kernel_ms_per_step": {k: round(x / max(vpn, 1), 5) for k, x in vkms.items() if x > 0}}
            v.close()

        if args.network:
            nr, nf = network_run(d, local, args.steps, flush, barrier)
            ref_f = base_at(nr["untimed_steps"] + args.steps)
            nr["rel_l2_vs_fp64"] = {f: float(np.linalg.norm(nf[f] - ref_f[f]) / np.linalg.norm(ref_f[f])) for f in ref_f}
            nr["precision_mode"], nr["warm_start"] = 3, 5
            nr["speedup_vs_fp64"] = nr["value"] / value
            variants["fp32_corrections_df_network"] = nr

    full = args.variants and args.variant_set == "all"
    ckpt = checkpoint_bench(d, local, barrier) if full else None
    c5 = metric_config_bench(args, local, flush, barrier) if full and args.c5_steps > 0 else None
    tb = blocking_ab(d, local, args.steps, flush, barrier, args.warm_lead) if full else None

    # the FP64 bit-exact path with the default launch shapes (no autotuning), beside the headline,
    # which uses the shapes the autotuner chose on the run's first steps (the shapes change no result)
    tuned = None
    if full:
        t = sts.Solver(d, fixed_sweeps=False, use_graph=True, device=local, precision=sts.EXACT, autotune=False)
        td, tms, tsw = timed_steps(t, args.steps, args.warmup, flush, barrier)
        tuned = {"value": Na * td * world / (tms / 1e3), "ms_per_step": tms / max(td, 1),
                 "sweeps_per_step": float(np.mean(tsw)) if len(tsw) else 0.0,
                 "launch_shapes": t.autotune_result()}
        t.close()

    if rank == 0:
        cpu = cpu_baseline(d, args.cpu_seconds, start_steps=0)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": done,
                "warmup": max(args.warmup, 3), "ms_per_step": total_ms / max(done, 1), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config(case, Nx, Ny), "roofline": roof, "cpu_baseline": cpu,
                "e2e": e2e, "clocks": clk.summary(), "gpu_launches": launches,
                "sweeps_per_step": {"mean": float(sum(sweeps) / max(len(sweeps), 1)),
                                    "max": int(max(sweeps)) if len(sweeps) else 0},
                "variants": variants,
                "warm_start_vs_plain": warm_summary(value, sweeps, variants),
                "checkpoint": ckpt, "untuned_fp64": tuned, "launch_shapes": launch_shapes,
                "metric_config": c5, "sweep_blocking_ab": tb}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
