"""Speed of the oracle port (oracle/kunoracle.c) against the reference's own
CPU executor (built from its sources by oracle/build_ref.py) on the same
inputs and thread count -- TEST INFRASTRUCTURE, run where the reference
sources are (not on the GPU machine, whose CPU baseline is the port).

    python oracle/port_speed.py [--stocks 2000] [--days 1000] [--threads N]

Prints one JSON line: per graph, seconds per run of each and the ratio
reference_time / port_time (above 1: the port is faster)."""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
# run as a script, the folder itself would shadow the oracle package
sys.path[:] = [p for p in sys.path if os.path.abspath(p or ".") != HERE]
sys.path.insert(0, os.path.dirname(HERE))


def _best(fn, reps):
    fn()
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return best


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--stocks", type=int, default=2000)
    ap.add_argument("--days", type=int, default=1000)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    from kunquant_gb300 import synth
    from kunquant_gb300.graph import predefined_spec
    from oracle import refkun
    from oracle.oracle import OracleProgram
    data = synth.ohlcv(args.stocks, args.days, seed=5, nan_frac=0.005)
    out = {"stocks": args.stocks, "days": args.days, "threads": args.threads}
    for key in ("alpha158_f32", "alpha101_f32"):
        prog = OracleProgram(predefined_spec(key))
        tp = _best(lambda: prog.run(data, nthreads=args.threads), args.reps)
        tr = _best(lambda: refkun.run_batch(key, data, threads=args.threads), args.reps)
        out[key] = {"port_s": tp, "reference_s": tr, "reference_over_port": tr / tp}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
