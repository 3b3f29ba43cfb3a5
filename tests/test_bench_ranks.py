"""The multi-replica path of bench.py on CPU ranks (gloo, world size 2):
the step time is the slowest rank's, the value counts every rank's
replica, and the reference arm prints from rank 0 only."""
import json
import os
import subprocess
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, q):
    sys.path.insert(0, REPO)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks([3.0, 7.5][rank], dist, "cpu")
    q.put((rank, ms, bench.job_value(world, 5000, 2500, ms)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_value_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    for _, ms, value in res:
        assert ms == 7.5
        assert value == pytest.approx(2 * 5000 * 2500 / 7.5e-3)


def test_reference_arm_prints_from_rank0_only(tmp_path):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    port = 30500 + os.getpid() % 1000
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--stocks", "200", "--days", "120"]
    r = subprocess.run(cmd, cwd=REPO, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0


def test_gpus_flag_launches_the_replicas_itself():
    """`bench.py --gpus 2` with no launcher starts two ranks by itself; the
    single line comes from rank 0 and counts both."""
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    env["CUDA_VISIBLE_DEVICES"] = ""
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--stocks", "200", "--days", "120"]
    r = subprocess.run(cmd, cwd=REPO, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    # n_gpus is the launched world size, read by the rank from WORLD_SIZE
    assert d["impl"] == "reference" and d["n_gpus"] == 2


def test_factor_errors_matches_numpy():
    """The GPU precision report's error measure, run on CPU tensors, equals
    the numpy form of the same definition."""
    import numpy as np
    import torch
    sys.path.insert(0, REPO)
    import bench
    rng = np.random.default_rng(5)
    w = rng.normal(size=(50, 40)) * 10
    g = w * (1 + rng.normal(size=w.shape) * 1e-6)
    w[3, 4] = np.nan
    g[7, 1] = np.nan
    w[9, 9] = 1e-9  # near zero: the floor applies
    got = bench._factor_errors({"f": torch.from_numpy(g.astype(np.float32))}, {"f": torch.from_numpy(w)})["f"]
    g32 = g.astype(np.float32).astype(np.float64)
    both = ~np.isnan(w) & ~np.isnan(g32)
    # torch's median of an even count is the lower middle value
    a = np.sort(np.abs(w[both]))
    m = a[(a.size - 1) // 2]
    rel = np.abs(g32[both] - w[both]) / np.maximum(np.abs(w[both]), 1e-3 * m + 1e-30)
    assert got[2] == 2
    assert got[0] == pytest.approx(rel.max(), rel=1e-12)
    assert got[1] == pytest.approx(np.sort(rel)[(rel.size - 1) // 2], rel=1e-12)


def test_clock_summary():
    """The clocks object of the bench line: median SM clock under load, the
    maximum, and every throttle reason seen active."""
    sys.path.insert(0, REPO)
    import bench
    rows = ["0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active\n",
            "0, 1950, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active\n",
            "0, 2040, 2070, 1200.0, 0x0, Not Active, Not Active, Not Active, Not Active\n",
            "garbage line\n"]
    c = bench.parse_clocks(rows)
    assert c == {"sm_mhz": 2040.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    assert bench.parse_clocks([]) is None


def test_stage_bytes_counts_distinct_series():
    """Algorithmic bytes of a stage: its distinct input and output series,
    each S x T elements."""
    sys.path.insert(0, REPO)
    import bench
    from kunquant_gb300.graph import predefined_spec
    spec = predefined_spec("alpha158_f32")
    for si, st in enumerate(spec["stages"]):
        n = len(set(st["in"]) | set(st["out"]))
        assert bench.stage_bytes(spec, si, 10, 20, 4) == n * 10 * 20 * 4
