"""Autotuner for the evaluator's launch configuration and scheduler (GPU).

The reference fixes its launch shape and work distribution at compile time
(src/hvm.cu:32-37 block and grid sizes, src/hvm.cu:116 bag length,
src/hvm.cu:1509-1548 the turn policy). Here they are runtime parameters, and
this module times a workload under each point of a small search space and
returns the fastest configuration:

  reg_cap_blocks  register cap of the turn kernel (0 = none, about 3 blocks of
                  128 threads per SM; 5 or 8 = that many blocks per SM)
  stack_cap       redexes per thread in the shared-memory deque
  graph_turns     0 = one launch per turn; k = CUDA-graph replays of k turns
  rule_select     0 = every lane interacts each round; 1 = one rule class per round
  fast_calls      CALL-time fast paths: 0 off, 1 SWITCH pattern, 2 SWITCH and ANNI
                  (compiled in for register caps 0, 5 and 8)
  policy          the fixed turn policy or the learned one

Every candidate's interaction count and results are checked against the first
candidate's (the configuration changes only the order of reduction).

    python lambdavm-rust_gb300/autotune.py --workload skewed_fold_2p18
"""
from __future__ import annotations

import argparse
import importlib
import itertools
import json
import math
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
hvm = importlib.import_module("lambdavm-rust_gb300")

DEFAULT_SPACE = {
    "reg_cap_blocks": (0, 5, 8),
    "stack_cap": (8, 16),
    "fast_calls": (0, 1),
    "policy": ("fixed", "learned"),
}


def candidates(space: dict | None = None) -> list[dict]:
    space = space or DEFAULT_SPACE
    keys = list(space)
    out = [dict(zip(keys, vals)) for vals in itertools.product(*(space[k] for k in keys))]
    # The fast-path kernel variants exist for register caps 0, 5 and 8.
    return [c for c in out if not (c.get("fast_calls") and c.get("reg_cap_blocks", 8) not in (0, 5, 8))]


def make_runtime(cand: dict, device: int = 0, weights=None, **extra):
    """A runtime configured as `cand` (its `policy` key selects the scheduler)."""
    cfg = {k: v for k, v in cand.items() if k != "policy"}
    rt = hvm.Runtime(device=device, **cfg, **extra)
    if cand.get("policy", "fixed") == "learned":
        if weights is None:
            weights = importlib.import_module("lambdavm-rust_gb300.train_policy").load_weights()
        rt.set_policy(hvm.POLICY_LEARNED, weights=weights)
    return rt


def tune_single(book, space: dict | None = None, reps: int = 2, device: int = 0, log=None):
    """Fastest configuration for one net: min wall time of `reps` evaluations.
    Returns (best candidate, rows of {candidate, ms})."""
    weights = importlib.import_module("lambdavm-rust_gb300.train_policy").load_weights()
    rows, want = [], None
    for cand in candidates(space):
        with make_runtime(cand, device, weights) as rt:
            rt.load(book)
            st = rt.run()  # warm-up, and the parity check
            got = (rt.result(), st.itrs)
            if want is None:
                want = got
            elif got != want:
                raise RuntimeError(f"configuration {cand} changed the result")
            best = math.inf
            for _ in range(reps):
                t0 = time.perf_counter()
                rt.run()
                best = min(best, (time.perf_counter() - t0) * 1e3)
        rows.append({"candidate": cand, "ms": best})
        if log:
            log(f"{cand} {best:.2f} ms")
    return min(rows, key=lambda r: r["ms"])["candidate"], rows


def tune_batch(books, max_inflight: int, live_frac: float, space: dict | None = None, reps: int = 1,
               device: int = 0, log=None):
    """Fastest configuration for a batch under continuous batching: min wall
    time of `reps` runs of the whole batch. Returns (best, rows)."""
    weights = importlib.import_module("lambdavm-rust_gb300.train_policy").load_weights()
    rows, want = [], None
    for cand in candidates(space):
        with make_runtime(cand, device, weights) as rt:
            rt.load_batch(books)
            st, _, res = rt.run_stream(max_inflight=max_inflight, live_frac=live_frac)  # warm-up
            got = (st.itrs, [int(p) for p in res])
            if want is None:
                want = got
            elif got != want:
                raise RuntimeError(f"configuration {cand} changed the batch's results")
            best = math.inf
            for _ in range(reps):
                t0 = time.perf_counter()
                rt.run_stream(max_inflight=max_inflight, live_frac=live_frac)
                best = min(best, time.perf_counter() - t0)
        rows.append({"candidate": cand, "seconds": best})
        if log:
            log(f"{cand} {best:.3f} s")
    return min(rows, key=lambda r: r["seconds"])["candidate"], rows


def main() -> None:
    W = importlib.import_module("lambdavm-rust_gb300.workloads")
    gens = {"bitonic_sort_2p16": lambda: W.bitonic_sort(16), "tree_sum_d20": lambda: W.tree_sum(20),
            "skewed_fold_2p18": lambda: W.skewed_fold(18), "countdown_30000": lambda: W.countdown(30000)}
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", choices=sorted(gens), default="skewed_fold_2p18")
    ap.add_argument("--reps", type=int, default=2)
    args = ap.parse_args()
    best, rows = tune_single(hvm.book_from_text(gens[args.workload]()), reps=args.reps, log=print)
    print(json.dumps({"workload": args.workload, "best": best}))


if __name__ == "__main__":
    main()
