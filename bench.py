"""Benchmark: Alpha158 fp32 factor-graph batch run (KunQuant runGraph) on GB300.

Workload (default): the Alpha158 factor graph (158 outputs from OHLCV+amount),
fp32, [T][S] layout, 5000 stocks x 2500 days of seeded synthetic OHLCV with
0.5% NaN cells.  One step = one runGraph over the whole batch.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  `value` is stock-days/s with the inputs resident on the
GPU; `e2e` is the same through the C ABI with pinned host buffers (host->device
inputs and device->host outputs inside the timed region).  The reference arm
(`--impl reference`) times the CPU restatement of the reference executor (the
oracle) on the host cores, on a bounded sample.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

WORKLOADS = {
    "alpha158": dict(key="alpha158_f32", module="alpha158", stocks=5000, days=2500, nan=0.005,
                     n_inputs=6, n_outputs=158),
    "alpha101": dict(key="alpha101_f32", module="alpha101", stocks=64, days=260, nan=0.0,
                     n_inputs=6, n_outputs=82),
    # the same graphs with the fast-stat rolling-moment accumulators
    "alpha158_fast": dict(key="alpha158_fast_f32", module="alpha158_fast", stocks=5000, days=2500, nan=0.005,
                          n_inputs=6, n_outputs=158),
    # fp32 factor arithmetic with the running sums in fp64
    "alpha158_acc64": dict(key="alpha158_acc64_f32", module="alpha158_acc64", stocks=5000, days=2500, nan=0.005,
                           n_inputs=6, n_outputs=158),
    # fp32 factor arithmetic with two-float compensated fp32 running sums
    "alpha158_comp": dict(key="alpha158_comp_f32", module="alpha158_comp", stocks=5000, days=2500, nan=0.005,
                          n_inputs=6, n_outputs=158),
    # Kahan fp32 window loops, two-float compensated rolling sums
    "alpha158_mixed": dict(key="alpha158_mixed_f32", module="alpha158_mixed", stocks=5000, days=2500, nan=0.005,
                           n_inputs=6, n_outputs=158),
    # the baseline form: one kernel launch per op, every value through HBM
    "alpha158_plain": dict(key="alpha158_plain_f32", module="alpha158_plain", stocks=5000, days=2500, nan=0.005,
                           n_inputs=6, n_outputs=158),
    "alpha101_fast": dict(key="alpha101_fast_f32", module="alpha101_fast", stocks=64, days=260, nan=0.0,
                          n_inputs=6, n_outputs=82),
    # window moments as two-float sliding window sums, scans in time chunks
    "alpha158_slide": dict(key="alpha158_slide_f32", module="alpha158_slide", stocks=5000, days=2500, nan=0.005,
                           n_inputs=6, n_outputs=158),
    "alpha101_slide": dict(key="alpha101_slide_f32", module="alpha101_slide", stocks=64, days=260, nan=0.0,
                           n_inputs=6, n_outputs=82),
    # the reference's own Alpha101 configuration: STs layout in and out
    "alpha101_sts": dict(key="alpha101_sts_f32", module="alpha101_sts", stocks=64, days=260, nan=0.0,
                         n_inputs=6, n_outputs=82),
}
# forms of the headline graph timed in the same run: the baseline (one
# launch per op) and the sliding-moment form
FORMS = {"alpha158": ["alpha158_plain", "alpha158_slide"]}


def max_over_ranks(ms: float, dist, device: str) -> float:
    """The slowest rank's step time (the whole job ends with it)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world: int, stocks: int, days: int, ms: float) -> float:
    """Whole-job stock-days/s: every rank runs its own replica of the
    workload (weak scaling), all done when the slowest one is."""
    return world * stocks * days / (ms / 1e3)


def relaunch_replicas(n: int) -> int:
    """`--gpus N` without a launcher: start N ranks of this same command
    under torch.distributed.run (one process per GPU, rendezvous on
    127.0.0.1); rank 0 prints the line.  Returns the launcher's exit code."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(n),
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd, cwd=REPO)


def _dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        with open(self.path) as f:
            lines = f.readlines()
        os.unlink(self.path)
        return parse_clocks(lines)


def parse_clocks(lines):
    """Summary of nvidia-smi rows (index, clocks.sm, clocks.max.sm, power,
    reasons.active, hw_slowdown, hw_thermal_slowdown, sw_thermal_slowdown,
    sw_power_cap): median SM clock, max clock and the throttle reasons seen
    active in any sample."""
    rows = []
    for line in lines:
        parts = [p.strip() for p in line.split(",")]
        if len(parts) >= 9:
            rows.append(parts)
    if not rows:
        return None
    sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
    mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
    reasons = set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for r in rows:
        for n, v in zip(names, r[5:9]):
            if v.lower() == "active":
                reasons.add(n)
    return {"sm_mhz": float(np.median(sm)) if sm else None,
            "sm_max_mhz": max(mx) if mx else None,
            "reasons": sorted(reasons), "samples": len(rows)}


def cpu_reference(workload: dict, steps: int, warmup: int, seconds_target: float = 15.0):
    """The reference executor's algorithm on the host cores (the oracle port),
    on a bounded sample of the workload: all stocks, a slice of the days."""
    from kunquant_gb300 import synth
    from kunquant_gb300.graph import predefined_spec
    from oracle.oracle import OracleProgram
    prog = OracleProgram(predefined_spec(workload["key"]))
    threads = os.cpu_count() or 1
    S = workload["stocks"]
    # calibrate the slice so a step takes a few seconds
    days = min(workload["days"], 100)
    data = synth.ohlcv(S, days, seed=7, nan_frac=workload["nan"])
    t0 = time.perf_counter()
    prog.run(data, nthreads=threads)
    dt = time.perf_counter() - t0
    per_sd = dt / (S * days)
    budget = seconds_target / max(1, steps + warmup)
    days = int(min(workload["days"], max(50, budget / per_sd / S)))
    data = synth.ohlcv(S, days, seed=7, nan_frac=workload["nan"])
    for _ in range(warmup):
        prog.run(data, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(steps):
        prog.run(data, nthreads=threads)
    dt = (time.perf_counter() - t0) / steps
    out = {"value": S * days / dt, "unit": "stock-days/s", "cores": threads, "kind": "port",
           "sample": f"{S} stocks x {days} days of the same seeded OHLCV, {steps} timed runs",
           "s_per_step": dt}
    # the port's speed against the reference executor itself, measured where
    # the reference sources are (oracle/port_speed.py)
    ps = os.path.join(REPO, "profiles", "cpu_port_vs_reference.json")
    if os.path.exists(ps):
        with open(ps) as f:
            rec = json.load(f)
        base = workload["key"].replace("_slide", "").replace("_plain", "")
        if base in rec:
            out["reference_over_port"] = {"value": rec[base]["reference_over_port"],
                                          "measured": f"{rec['host']}, {rec['threads']} threads, "
                                                      f"{rec['stocks']} x {rec['days']}",
                                          "source": "profiles/cpu_port_vs_reference.md"}
    return out


def serving(nsess=256, rate=20000.0, seconds=3.0, warm=250, seed=3):
    """Stream serving of the Alpha101 stream module: `nsess` sessions of
    log-uniform size in [100, 5000] stocks in one pool, each warmed with
    `warm` days of history.  Bars then arrive as a Poisson process at an
    aggregate `rate` session-ticks/s (each to a session drawn uniformly);
    a session with a tick in flight queues its next bar.  The request loop
    batches whatever is submitted while a step runs.  Latency is arrival to
    result in the pinned host table.  For contrast, the same ticks through one
    StreamContext per session, called one after another."""
    from collections import deque
    from kunquant_gb300 import runner as kr
    from kunquant_gb300 import serve
    mod = kr.Library.predefined("alpha101_stream_f32").getModule("alpha101_stream")
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(100), np.log(5000), nsess)).astype(int)
    cap = int(sizes.sum())
    ex = kr.createSingleThreadExecutor()
    pool = serve.ServePool(ex, mod, capacity_stocks=cap, max_sessions=nsess, max_session_stocks=5000)
    sess = [pool.open(int(n)) for n in sizes]
    names = mod.getInputNames()
    base = rng.uniform(10, 100, cap).astype(np.float32)
    day = [0] * nsess

    def write(i):
        s = sess[i]
        row = base[s.column:s.column + s.num_stocks] * np.float32(1 + 0.001 * (day[i] % 100))
        for k in names:
            s.inputs[k][:] = row
        day[i] += 1

    # history: every session steps through `warm` days together
    for _ in range(warm):
        for i in range(nsess):
            write(i)
        pool.submit_all(sess)
        for s in sess:
            s.wait(60000)
    pool.take_latencies()
    # Poisson arrivals
    n_arr = int(rate * seconds)
    arr_t = np.cumsum(rng.exponential(1.0 / rate, n_arr))
    arr_s = rng.integers(0, nsess, n_arr)
    pending = [deque() for _ in range(nsess)]
    inflight, waiting = {}, set()
    lat = []
    i = 0
    t0 = time.perf_counter()
    while i < n_arr or inflight or waiting:
        now = time.perf_counter() - t0
        while i < n_arr and arr_t[i] <= now:
            j = int(arr_s[i])
            pending[j].append(arr_t[i])
            if j not in inflight:
                waiting.add(j)
            i += 1
        done = [j for j in inflight if sess[j].ticks >= sess[j]._submitted]
        if done:
            tdone = time.perf_counter() - t0
            for j in done:
                lat.append(tdone - inflight.pop(j))
                if pending[j]:
                    waiting.add(j)
        if waiting:
            batch = list(waiting)
            waiting.clear()
            for j in batch:
                write(j)
                inflight[j] = pending[j].popleft()
            pool.submit_all([sess[j] for j in batch])
    el = time.perf_counter() - t0
    # the pool's own record: submit to result, per tick (without the
    # harness's arrival queue and polling)
    native, steps = pool.take_latencies()
    pool.shutdown()
    lat = np.asarray(lat) * 1e6
    # the same kind of tick through one StreamContext per session, one call after another
    k = min(32, nsess)
    ctxs = [kr.StreamContext(ex, mod, int(sizes[j])) for j in range(k)]
    hs = [{n: c.queryBufferHandle(n) for n in names} for c in ctxs]
    rows = [base[:int(sizes[j])] for j in range(k)]
    for rep in range(3):
        if rep == 1:
            tp = time.perf_counter()
        for c, h, r in zip(ctxs, hs, rows):
            for n in names:
                c.pushData(h[n], r)
            c.run()
    per_call = (time.perf_counter() - tp) / (2 * k)
    return {"module": "alpha101_stream_f32", "sessions": nsess, "stocks": cap,
            "sizes": "log-uniform [100, 5000] stocks per session", "history_days": warm,
            "arrivals": f"Poisson, {rate:.0f} session-ticks/s aggregate, {seconds:.0f} s",
            "ticks": int(lat.size), "p50_tick_us": float(np.percentile(lat, 50)),
            "p99_tick_us": float(np.percentile(lat, 99)), "session_ticks_per_s": lat.size / el,
            "stock_ticks_per_s": float(lat.size / el * sizes.mean()),
            "mean_sessions_per_step": float(np.mean(steps)) if len(steps) else None,
            "pool_submit_to_result_us": {"p50": float(np.percentile(native, 50)) if len(native) else None,
                                         "p99": float(np.percentile(native, 99)) if len(native) else None},
            "pool_bytes": serve.pool_bytes(mod, cap),
            "one_context_per_session": {"ms_per_session_tick": per_call * 1e3,
                                        "max_session_ticks_per_s": 1.0 / per_call}}


def serve_steps_main(args):
    """Serving steps driven by the caller (no request loop): `--sessions`
    sessions of the Alpha101 stream module (sizes log-uniform in [100, 5000],
    the serving workload's first ones) advance one tick together per step;
    CUDA-event time per step after `--warmup` steps."""
    import torch
    from kunquant_gb300 import runner as kr
    from kunquant_gb300 import serve
    torch.cuda.set_device(0)
    mod = kr.Library.predefined("alpha101_stream_f32").getModule("alpha101_stream")
    rng = np.random.default_rng(3)
    sizes = np.exp(rng.uniform(np.log(100), np.log(5000), 256)).astype(int)[:args.sessions]
    cap = int(sizes.sum())
    ex = kr.createSingleThreadExecutor()
    pool = serve.ServePool(ex, mod, capacity_stocks=cap, max_sessions=256, max_session_stocks=5000, start=False)
    sess = [pool.open(int(k)) for k in sizes]
    for s in sess:
        for k in mod.getInputNames():
            s.inputs[k][:] = rng.uniform(10, 100, s.num_stocks).astype(np.float32)
    for _ in range(args.warmup):
        pool.step(sess)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pool.step(sess)
    dt = (time.perf_counter() - t0) / args.steps
    pool.shutdown()
    print(json.dumps({"metric": "ms per serving step", "value": dt * 1e3, "unit": "ms", "higher_is_better": False,
                      "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "data": "synthetic",
                      "config": {"workload": f"alpha101_stream_f32 serving step, {args.sessions} sessions, "
                                             f"{cap} stocks, caller-driven (kunServeStep)"}}))


def universes_main(args):
    """Many universes of uneven size: `--universes` universes of Alpha158 fp32
    with S log-uniform in [37, 6000] stocks and T uniform in [250, 5000] days
    (seeded), every other one also running Alpha101 fp32.  A step is one
    kunRunGraphBatch per module over its universes; against it, one runGraph
    per (universe, module) on the same executor."""
    import torch
    from kunquant_gb300 import runner as kr
    from kunquant_gb300 import synth
    torch.cuda.set_device(0)
    rng = np.random.default_rng(4242)
    n = args.universes
    Ss = np.exp(rng.uniform(np.log(37), np.log(6000), n)).astype(int)
    Ts = rng.integers(250, 5001, n)
    mods = {"alpha158": kr.Library.predefined("alpha158_f32").getModule("alpha158"),
            "alpha101": kr.Library.predefined("alpha101_f32").getModule("alpha101")}
    members = {"alpha158": list(range(n)), "alpha101": list(range(0, n, 2))}
    ins = []
    for i in range(n):
        d = synth.ohlcv(int(Ss[i]), int(Ts[i]), seed=1000 + i, nan_frac=0.005)
        ins.append({k: torch.from_numpy(v).cuda() for k, v in d.items()})
    outs = {m: [{k: torch.empty((int(Ts[i]), int(Ss[i])), device="cuda") for k in mods[m].getOutputNames()}
                for i in members[m]] for m in mods}
    units = {m: float(sum(int(Ss[i]) * int(Ts[i]) for i in members[m])) for m in mods}
    ex = kr.createSingleThreadExecutor()
    tuned = {m: 0 if args.no_tune else kr.tune(ex, mods[m], [ins[i] for i in members[m]], reps=2) for m in mods}

    def batched(ms=tuple(mods)):
        def run():
            for m in ms:
                kr.runGraphBatch(ex, mods[m], [ins[i] for i in members[m]], outputs_list=outs[m])
        return run

    def one_by_one():
        for m in mods:
            for j, i in enumerate(members[m]):
                kr.runGraph(ex, mods[m], ins[i], 0, int(Ts[i]), outputs=outs[m][j])

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    ms_158 = timed(batched(("alpha158",)))
    launches_158 = ex.last_launch_count()
    ms_b = timed(batched())
    launches = launches_158 + ex.last_launch_count()  # the step's second call is alpha101's
    ms_s = timed(one_by_one)
    total = sum(units.values())
    line = {"metric": "stock-days/s", "value": total / (ms_b / 1e3), "unit": "stock-days/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_b, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{n} universes of alpha158 fp32 TS (every other one also alpha101), "
                                   f"S log-uniform [37, 6000], T uniform [250, 5000], 0.5% NaN cells",
                       "stock_days": units, "autotuned_stages": tuned,
                       "l2": "inputs exceed the 129 MB L2; no flush"},
            "gpu_launches": launches,
            "alpha158_only": {"value": units["alpha158"] / (ms_158 / 1e3), "ms_per_step": ms_158,
                              "gpu_launches": launches_158},
            "one_runGraph_per_universe_and_module": {"value": total / (ms_s / 1e3), "ms_per_step": ms_s}}
    print(json.dumps(line))


PRECISION_FORMS = {
    "alpha158": ["alpha158_f32", "alpha158_fast_f32", "alpha158_mixed_f32", "alpha158_comp_f32",
                 "alpha158_acc64_f32", "alpha158_slide_f32"],
    "alpha101": ["alpha101_f32", "alpha101_mixed_f32", "alpha101_comp_f32", "alpha101_acc64_f32",
                 "alpha101_slide_f32"],
}


def _factor_errors(got, want):
    """Per factor (max rel err, median rel err, NaN cells that differ) of a
    fp32 form against the fp64 build, on the GPU.  The relative error is
    |got - want| / max(|want|, 1e-3 * median |want|) over cells where both
    are numbers (the floor keeps values crossing zero from dividing by ~0)."""
    import torch
    out = {}
    for k, w in want.items():
        g = got[k].double()
        gn, wn = torch.isnan(g), torch.isnan(w)
        nanmis = int((gn != wn).sum())
        both = ~gn & ~wn
        if bool(both.any()):
            wb, gb = w[both], g[both]
            m = wb.abs().median()
            rel = (gb - wb).abs() / torch.clamp(wb.abs(), min=float(1e-3 * m + 1e-30))
            out[k] = (float(rel.max()), float(rel.median()), nanmis)
        else:
            out[k] = (0.0, 0.0, nanmis)
    return out


def precision_main(args):
    """Per-factor error of the fp32 forms (exact fp32, fast-stat, two-float
    compensated sums, fp64 sums) against the fp64 build, on Alpha158 and
    Alpha101 over S x T cells of seeded OHLCV whose price levels are drawn
    log-uniform in [1, 1e5].  The fp64 build is the truth: it reproduces the
    reference's fp64 TS build bit for bit (the fp64 parity tests)."""
    import torch
    from kunquant_gb300 import runner as kr
    from kunquant_gb300 import synth
    torch.cuda.set_device(0)
    S, T = args.stocks or 8192, args.days or 4000
    d32 = synth.ohlcv(S, T, seed=77, nan_frac=0.0, price_range=(1.0, 1e5))
    in32 = {k: torch.from_numpy(v).cuda() for k, v in d32.items()}
    in64 = {k: v.double() for k, v in in32.items()}
    ex = kr.createSingleThreadExecutor()
    summary, tables = {}, []
    for graph, forms in PRECISION_FORMS.items():
        m64 = kr.Library.predefined(f"{graph}_f64").getModule(f"{graph}_f64")
        want = kr.runGraph(ex, m64, in64, 0, T)
        stats = {}
        for key in forms:
            name = key[:-4]
            mod = kr.Library.predefined(key).getModule(name)
            got = kr.runGraph(ex, mod, in32, 0, T)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            kr.runGraph(ex, mod, in32, 0, T, outputs=got)
            e1.record()
            torch.cuda.synchronize()
            st = stats[name] = _factor_errors(got, want)
            del got
            med = [v[1] for v in st.values()]
            summary[name] = {"factors": len(st), "max_le_1e-5": sum(v[0] <= 1e-5 for v in st.values()),
                             "median_le_1e-5": sum(m <= 1e-5 for m in med),
                             "worst_median": max(med), "nan_cells_differing": sum(v[2] for v in st.values()),
                             "ms": e0.elapsed_time(e1)}
        del want
        torch.cuda.empty_cache()
        names = sorted(next(iter(stats.values())))
        tables.append(f"## {graph}\n\n| factor | " + " | ".join(f"{n} max | {n} median | {n} NaN diff" for n in stats)
                      + " |\n|---|" + "---|---|---|" * len(stats))
        for f in names:
            tables.append(f"| {f} | " + " | ".join(f"{stats[n][f][0]:.1e} | {stats[n][f][1]:.1e} | {stats[n][f][2]}"
                                                  for n in stats) + " |")
        tables.append("")
    if args.report:
        with open(args.report, "w") as f:
            f.write(f"# fp32 forms vs the fp64 build, {S} stocks x {T} days, prices log-uniform in [1, 1e5]\n\n")
            for n, v in summary.items():
                f.write(f"- {n}: {json.dumps(v)}\n")
            f.write("\n" + "\n".join(tables))
    line = {"metric": "factors with median rel err <= 1e-5", "value": summary["alpha158_comp"]["median_le_1e-5"],
            "unit": "factors", "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"precision: alpha158 + alpha101, {S} stocks x {T} days, price levels "
                                   f"log-uniform in [1, 1e5], truth = the fp64 build"},
            "forms": summary}
    print(json.dumps(line))


def stage_bytes(mod_spec, stage_idx, S, T, elem):
    st = mod_spec["stages"][stage_idx]
    return (len(set(st["in"])) + len(st["out"])) * S * T * elem


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="alpha158",
                    choices=sorted(WORKLOADS) + ["universes", "precision", "serve_steps"])
    ap.add_argument("--sessions", type=int, default=16, help="sessions of the 'serve_steps' workload")
    ap.add_argument("--report", default=None, help="precision workload: write the per-factor table here")
    ap.add_argument("--stocks", type=int, default=None)
    ap.add_argument("--days", type=int, default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serve", action="store_true", help="skip the stream-serving measurement")
    ap.add_argument("--no-tune", action="store_true", help="keep the generated launch shapes (no autotuning)")
    ap.add_argument("--no-forms", action="store_true", help="skip timing the plain and slide forms")
    ap.add_argument("--universes", type=int, default=48, help="universes of the 'universes' workload")
    ap.add_argument("--streams", type=int, default=8, help="CUDA streams for concurrent stages")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_replicas(args.gpus))
    if args.workload == "serve_steps":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "serve_steps times the GPU serving pool only"}))
            return
        return serve_steps_main(args)
    if args.workload == "precision":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the precision workload compares the GPU forms "
                              "with each other; the reference arm times the batch workloads"}))
            return
        return precision_main(args)
    if args.workload == "universes":
        if args.impl == "reference":
            args.workload = "alpha158"  # the CPU arm times the same graph per stock-day
        else:
            return universes_main(args)
    wl = dict(WORKLOADS[args.workload])
    if args.stocks:
        wl["stocks"] = args.stocks
    if args.days:
        wl["days"] = args.days
    world, rank, local = _dist_env()
    config = {"workload": f"{args.workload} fp32 TS, {wl['stocks']} stocks x {wl['days']} days, "
                          f"{wl['nan'] * 100:.1f}% NaN cells",
              "module": wl["key"], "stocks": wl["stocks"], "days": wl["days"],
              "l2": "inputs (6 x S x T x 4 B) exceed the 129 MB L2; no flush"}
    metric = "stock-days/s"
    if args.impl == "reference":
        if rank != 0:
            return
        ref = cpu_reference(wl, args.steps, args.warmup)
        line = {"metric": metric, "value": ref["value"], "unit": "stock-days/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ref["s_per_step"] * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": config, "impl": "reference",
                "cpu_baseline": {k: ref[k] for k in ("value", "unit", "cores", "kind", "sample",
                                                     "reference_over_port") if k in ref},
                "e2e": {"value": ref["value"], "unit": "stock-days/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    from kunquant_gb300 import runner as kr
    from kunquant_gb300 import synth
    from kunquant_gb300.graph import predefined_spec
    spec = predefined_spec(wl["key"])
    S, T = wl["stocks"], wl["days"]
    lib = kr.Library.predefined(wl["key"])
    mod = lib.getModule(wl["module"])
    data = synth.ohlcv(S, T, seed=1234 + rank, nan_frac=wl["nan"])
    dev_in = {k: torch.from_numpy(v).cuda() for k, v in data.items()}
    dev_out = {n: torch.empty((T, S), dtype=torch.float32, device="cuda") for n in mod.getOutputNames()}
    ex = kr.createMultiThreadExecutor(args.streams)
    tuned = 0
    if not args.no_tune:
        # the autotuner times candidate launch shapes of every stage on this
        # workload (untimed, like a compilation step)
        tuned = kr.tune(ex, mod, [dev_in], reps=2)
    config["autotuned_stages"] = tuned

    def step():
        kr.runGraph(ex, mod, dev_in, 0, T, outputs=dev_out)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    launches = 0
    for _ in range(args.steps):
        step()
        launches += ex.last_launch_count()
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    ms_step = e0.elapsed_time(e1) / args.steps
    # per-stage kernel time: a profiled single-stream pass over the same data
    # (CUDA events after every stage launch on the launching stream)
    ex.set_profiling(True)
    stage_ms = {}
    for _ in range(2):
        step()
        for sid, ms in ex.stage_times():
            stage_ms.setdefault(sid, []).append(ms)
    ex.set_profiling(False)
    ms_step = max_over_ranks(ms_step, dist, "cuda")
    value = job_value(world, S, T, ms_step)

    # dominant kernel and its HBM roofline
    avg = {sid: float(np.mean(v)) for sid, v in stage_ms.items()}
    top = max(avg, key=avg.get)
    elem = 4
    alg_bytes = stage_bytes(spec, top, S, T, elem)
    achieved = alg_bytes / (avg[top] / 1e3) / 1e9
    peak, peak_kind = _peaks()
    # DRAM traffic of the stage is not measured in this run (an ncu capture
    # of the same tuned launch shapes would be needed); per-kernel captures
    # are in profiles/
    traffic = None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                "kernel": f"stage {top} of {wl['key']} ({avg[top]:.3f} ms/launch, "
                          f"{100 * avg[top] / sum(avg.values()):.1f}% of kernel time, single-stream profiled pass)",
                "whole_step_frac": (wl["n_inputs"] + wl["n_outputs"]) * S * T * elem / (ms_step / 1e3) / 1e9 / peak}

    # the other forms of the same graph on the same inputs and executor
    forms = None
    if not args.no_forms and args.workload in FORMS:
        forms = {}
        for fw in FORMS[args.workload]:
            fk = WORKLOADS[fw]
            fmod = kr.Library.predefined(fk["key"]).getModule(fk["module"])
            ftuned = 0 if args.no_tune else kr.tune(ex, fmod, [dev_in], reps=2)

            def fstep():
                kr.runGraph(ex, fmod, dev_in, 0, T, outputs=dev_out)

            for _ in range(args.warmup):
                fstep()
            torch.cuda.synchronize()
            f0 = torch.cuda.Event(enable_timing=True)
            f1 = torch.cuda.Event(enable_timing=True)
            f0.record(stream)
            flaunch = 0
            for _ in range(args.steps):
                fstep()
                flaunch += ex.last_launch_count()
            f1.record(stream)
            torch.cuda.synchronize()
            fms = max_over_ranks(f0.elapsed_time(f1) / args.steps, dist, "cuda")
            forms[fw] = {"ms_per_step": fms, "value": job_value(world, S, T, fms), "autotuned_stages": ftuned,
                         "gpu_launches": flaunch}
        if "alpha158_plain" in forms:
            for fw in forms:
                forms[fw]["over_plain"] = forms["alpha158_plain"]["ms_per_step"] / forms[fw]["ms_per_step"]
            forms["alpha158"] = {"ms_per_step": ms_step, "value": value,
                                 "over_plain": forms["alpha158_plain"]["ms_per_step"] / ms_step}

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        host_in = {k: torch.from_numpy(v).pin_memory().numpy() for k, v in data.items()}
        host_out = {n: torch.empty((T, S), dtype=torch.float32).pin_memory().numpy()
                    for n in mod.getOutputNames()}
        for _ in range(max(1, args.warmup)):
            kr.runGraph(ex, mod, host_in, 0, T, outputs=host_out)
        step_ms = []
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ts = time.perf_counter()
            kr.runGraph(ex, mod, host_in, 0, T, outputs=host_out)
            step_ms.append((time.perf_counter() - ts) * 1e3)
        dt = (time.perf_counter() - t0) / args.steps
        e2e = {"value": world * S * T / dt, "unit": "stock-days/s",
               "h2d_bytes_per_step": wl["n_inputs"] * S * T * elem,
               "d2h_bytes_per_step": len(host_out) * S * T * elem, "ms_per_step": dt * 1e3,
               "step_ms_median": float(np.median(step_ms)), "step_ms_max": max(step_ms)}
    serve_line = None
    if rank == 0 and not args.no_serve:
        serve_line = serving()
    cpu = None
    if rank == 0 and not args.no_cpu:
        ref = cpu_reference(wl, 2, 1, seconds_target=12.0)
        cpu = {k: ref[k] for k in ("value", "unit", "cores", "kind", "sample", "reference_over_port") if k in ref}
    if rank == 0:
        line = {"metric": metric, "value": value, "unit": "stock-days/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": config, "roofline": roofline, "cpu_baseline": cpu,
                "serving": serve_line, "forms": forms,
                "e2e": e2e, "gpu_launches": launches, "clocks": clocks,
                "stage_ms": {str(k): round(v, 4) for k, v in sorted(avg.items(), key=lambda x: -x[1])[:8]}}
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
