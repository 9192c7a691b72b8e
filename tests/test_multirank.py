"""The multi-rank path of bench.py on CPU (gloo, world size 2): every rank advances its own
replica of the case (no collective on the data path), the job's time is the slowest rank's,
the throughput counts every rank's cells, and the reference arm runs on rank 0 only."""
import os
import socket
import tempfile

import numpy as np
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def worker(rank, world, port, out_dir):
    import sys
    sys.path[:0] = [ROOT, os.path.join(ROOT, "simple-ts_gb300"), os.path.join(ROOT, "oracle")]
    import torch.distributed as dist
    import bench
    import ora
    import sts_cases as sc
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    # each rank: its own replica of the same case, stepped independently
    d = tempfile.mkdtemp()
    sc.channel_case("c", 40, 6, 0.3, 0.002, 1e-3, 20).write(d)
    o = ora.Oracle(d, fixed_sweeps=False)
    steps = o.step(3)
    ms = 10.0 + 5.0 * rank  # rank 1 is the slower one
    job_ms = bench.slowest(ms, world, device="cpu")
    rate = bench.job_rate(o.Nx * o.Ny * steps, world, job_ms / 1e3)
    np.save(os.path.join(out_dir, f"p{rank}.npy"), o.field("p"))
    with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
        f.write(f"{job_ms} {rate} {o.Nx * o.Ny * steps}")
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_and_slowest_rank_timing(oracle_built):
    port = free_port()
    with tempfile.TemporaryDirectory() as out:
        mp.start_processes(worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
        vals = [open(os.path.join(out, f"r{r}.txt")).read().split() for r in range(2)]
        job_ms = [float(v[0]) for v in vals]
        rates = [float(v[1]) for v in vals]
        cells = int(vals[0][2])
        assert job_ms == [15.0, 15.0]          # both ranks see the slowest rank's time
        assert rates[0] == rates[1] == cells * 2 / 0.015
        np.testing.assert_array_equal(np.load(os.path.join(out, "p0.npy")), np.load(os.path.join(out, "p1.npy")))


def test_reference_arm_runs_on_rank_zero_only(capsys, monkeypatch):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        workload = "channel_ma2.43"
        warmup = 1
        steps = 1
        gpus = 2
    assert bench.reference_arm(Args()) is None
    assert capsys.readouterr().out == ""


def test_partition_covers_every_case_once():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    cells = bench.batch_cells()
    assert len(cells) == 64
    for world in (1, 2, 3, 4, 8):
        parts = bench.partition_cases(cells, world)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(64))
        loads = [sum(cells[k] for k in p) for p in parts]
        assert max(loads) - min(loads) <= max(cells)  # greedy largest-first balance
        assert parts == bench.partition_cases(cells, world)  # every rank computes the same


def shard_worker(rank, world, port, out_dir):
    import sys
    sys.path[:0] = [ROOT, os.path.join(ROOT, "simple-ts_gb300"), os.path.join(ROOT, "oracle")]
    import torch.distributed as dist
    import bench
    import ora
    import sts_cases as sc
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    cases = sc.batch_cases(n=6, Nt=10, nx_range=(30, 60))
    mine = bench.partition_cases([c.Nx * c.Ny for c in cases], world)[rank]
    for k in mine:  # each rank advances only its own cases
        d = tempfile.mkdtemp()
        cases[k].write(d)
        o = ora.Oracle(d, fixed_sweeps=False)
        o.step(3)
        np.save(os.path.join(out_dir, f"case{k}_rank{rank}.npy"), np.stack([o.field(f) for f in ("u", "v", "p", "T")]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_case_sharding_equals_single_process(oracle_built):
    """Sharded over two gloo ranks, every case is advanced by exactly one rank, and its fields
    equal those of the same case advanced in a single process."""
    import sys
    sys.path[:0] = [os.path.join(ROOT, "simple-ts_gb300"), os.path.join(ROOT, "oracle")]
    import ora
    import sts_cases as sc
    port = free_port()
    with tempfile.TemporaryDirectory() as out:
        mp.start_processes(shard_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
        files = sorted(os.listdir(out))
        owners = {}
        for f in files:
            k = int(f.split("_")[0][4:])
            owners.setdefault(k, []).append(f)
        assert sorted(owners) == list(range(6)) and all(len(v) == 1 for v in owners.values())
        for k, c in enumerate(sc.batch_cases(n=6, Nt=10, nx_range=(30, 60))):
            with tempfile.TemporaryDirectory() as d:
                c.write(d)
                o = ora.Oracle(d, fixed_sweeps=False)
                o.step(3)
                want = np.stack([o.field(f) for f in ("u", "v", "p", "T")])
            np.testing.assert_array_equal(np.load(os.path.join(out, owners[k][0])), want)
