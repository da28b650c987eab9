"""Trains the turn scheduler's MLP from evaluator traces (GPU).

The reference schedules turns with a fixed SEED/GROW/WORK policy
(src/hvm.cu:1509-1548); this runtime's fixed policy is its counterpart and the
learned policy is trained on decisions that measured faster:

1. Labels (default, `--labels search`): every training net runs under the
   fixed policy with per-turn tracing; then, for each turn k, each candidate
   decision (budget, stop fraction) is applied at the close of turn k alone
   (POLICY_SCRIPT; the fixed policy decides every other turn from the state it
   meets) and the run timed. The fastest decision labels turn k's 16 features
   when it beats the fixed run by 2 %; otherwise the fixed decision does.
   (`--labels constant`: the best of a grid of constant schedules per net
   labels all of that net's turns.)
2. Each net's turns are weighted equally.
3. The MLP is trained on the GPU (hvm_gb300_policy_train: full-batch Adam, one
   CUDA-graph replay per epoch) and written to a JSON file with the per-net
   timings of the fixed and learned schedules.

Normal forms and interaction counts are the same under every schedule; each
run is checked against the fixed policy's.

    python lambdavm-rust_gb300/train_policy.py --out lambdavm-rust_gb300/policy_weights.json
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

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
hvm = importlib.import_module("lambdavm-rust_gb300")
wl = importlib.import_module("lambdavm-rust_gb300.workloads")

# Constant schedules: (budget, stop fraction, share) per regime; -1 keeps the
# fixed policy's choice.
SEED_BUDGET = (-1.0, 0.0, 0.4, 1.0)
WORK_BUDGET = (-1.0, 0.6)
WORK_STOP = (-1.0, 0.25, 0.5)
WORK_SHARE = (-1.0, 0.5)


def constant_grid() -> list[tuple[float, ...]]:
    grid = []
    for sb, wb, ws, wsh in itertools.product(SEED_BUDGET, WORK_BUDGET, WORK_STOP, WORK_SHARE):
        grid.append((sb, -1.0, -1.0, wb, ws, wsh))
    return grid


def training_streams(n: int = 768) -> list[tuple[str, list[str]]]:
    """Continuously batched streams: two slices of the 4096-net mixed pool
    (the batch benchmark runs the whole pool)."""
    pool = wl.mixed_batch(4096)
    return [(f"stream_{n}_a", [c for c, _ in pool[:n]]), (f"stream_{n}_b", [c for c, _ in pool[2048:2048 + n]])]


def training_nets() -> list[tuple[str, str]]:
    """Seeded nets of the benchmark families, none equal to a benchmark input."""
    nets = []
    for k, (lg, p) in enumerate(itertools.product((12, 14, 16), (1 / 16, 1 / 64, 1 / 256))):
        seed = 0x5EED0000 + k
        nets.append((f"skewed_fold_2p{lg}_p{round(1 / p)}", wl.skewed_fold(lg, seed=seed, p=p)))
    for d in (14, 17):
        nets.append((f"tree_sum_d{d}", wl.tree_sum(d)))
    for lg in (10, 12):
        nets.append((f"bitonic_sort_2p{lg}_s", wl.bitonic_sort(lg, seed=0xB170 + lg)))
    for n in (3000, 30000):
        nets.append((f"countdown_{n}", wl.countdown(n)))
    return nets


# Continuous-batching settings of the batch benchmark.
STREAM_INFLIGHT, STREAM_LIVE_FRAC = 512, 0.25


def timed_run(rt, reps: int, stream: bool = False) -> tuple[float, object]:
    """Best time (ms) over `reps` runs, and the last run's stats: device time
    for a single net, wall time for a stream (admission is part of it)."""
    best, st = math.inf, None
    for _ in range(reps):
        rt.reset_counters()
        if stream:
            t0 = time.perf_counter()
            st, _, res = rt.run_stream(max_inflight=STREAM_INFLIGHT, live_frac=STREAM_LIVE_FRAC)
            best = min(best, (time.perf_counter() - t0) * 1e3)
            st.results = tuple(int(p) for p in res)
        else:
            st = rt.run()
            best = min(best, st.kernel_ms)
    return best, st


def _load(rt, item) -> bool:
    """Loads a single net (text) or a stream (list of texts); True for a stream."""
    if isinstance(item, list):
        rt.load_batch([hvm.book_from_text(c) for c in item])
        return True
    rt.load(item)
    return False


def _outcome(rt, st, stream: bool):
    return (st.results, st.itrs) if stream else (rt.result(), st.itrs)


def collect(nets, reps: int, trace_cap: int, log=print):
    grid = constant_grid()
    xs, ts, ws, report = [], [], [], []
    for name, code in nets:
        with hvm.Runtime(device=0, trace_cap=trace_cap) as rt:
            stream = _load(rt, code)
            rt.set_policy(hvm.POLICY_FIXED)
            fixed_ms, st0 = timed_run(rt, reps, stream)
            want = _outcome(rt, st0, stream)
            best = (fixed_ms, None, rt.trace())
            for const in grid:
                rt.set_policy(hvm.POLICY_CONSTANT, constants=const)
                ms, st = timed_run(rt, reps, stream)
                if _outcome(rt, st, stream) != want:
                    raise RuntimeError(f"{name}: schedule {const} changed the result")
                if ms < best[0]:
                    best = (ms, const, rt.trace())
            ms, const, trace = best
            feats = np.array([r["features"] for r in trace], dtype=np.float32)
            outs = np.array([r["outputs"] for r in trace], dtype=np.float32)
            # The last record closes the final turn: nothing follows it.
            feats, outs = feats[:-1], outs[:-1]
            if len(feats):
                xs.append(feats)
                ts.append(np.clip(outs, 0.0, 1.0))
                ws.append(np.full(len(feats), 1.0 / len(feats), dtype=np.float32))
            report.append({"net": name, "itrs": want[1], "fixed_ms": round(fixed_ms, 3),
                           "best_ms": round(ms, 3), "best_schedule": const, "turns": len(trace)})
            log(f"{name:28s} itrs={want[1]:>11d} fixed={fixed_ms:8.2f} ms best={ms:8.2f} ms {const}")
    return np.concatenate(xs), np.concatenate(ts), np.concatenate(ws), report


# Candidate decisions for the per-turn search (output space: budget 64 << 10 o0
# rounds -- 64, 256, 512, 1024, the default turn cap --, stop fraction; the
# static share keeps the fixed policy's choice).
SEARCH_ACTIONS = tuple((b, f, -1.0) for b in (0.0, 0.2, 0.3, 0.4) for f in (0.0, 0.5))


def search(nets, reps: int, trace_cap: int, max_turns: int = 48, margin: float = 0.02, log=print):
    """Per-decision labels by local search: for each turn k of a net's run
    under the fixed policy, every candidate decision is tried at the close of
    turn k alone (the fixed policy decides every other turn, from the state it
    then meets), and the fastest run labels turn k's features -- when it beats
    the fixed run by `margin`, else the fixed policy's own decision is the
    label. Device time, best of `reps`; every run is checked against the
    fixed run's normal form and interaction count."""
    xs, ts, ws, report = [], [], [], []
    for name, code in nets:
        if isinstance(code, list):
            continue  # streams: a run is seconds long, too long to search turn by turn
        with hvm.Runtime(device=0, trace_cap=trace_cap) as rt:
            rt.load(code)
            rt.set_policy(hvm.POLICY_FIXED)
            fixed_ms, st0 = timed_run(rt, reps)
            want = _outcome(rt, st0, False)
            trace = rt.trace()
            turns = min(len(trace) - 1, max_turns)
            feats, labels, moved = [], [], 0
            for k in range(turns):
                best_ms, best = fixed_ms * (1.0 - margin), None
                for act in SEARCH_ACTIONS:
                    rt.set_policy(hvm.POLICY_SCRIPT, weights=[-1.0] * (3 * k) + list(act))
                    ms, st = timed_run(rt, reps)
                    if _outcome(rt, st, False) != want:
                        raise RuntimeError(f"{name}: decision {act} at turn {k} changed the result")
                    if ms < best_ms:
                        best_ms, best = ms, act
                feats.append(trace[k]["features"])
                out = list(trace[k]["outputs"]) if best is None else [best[0], best[1], trace[k]["outputs"][2]]
                labels.append(out)
                moved += best is not None
            if feats:
                xs.append(np.array(feats, dtype=np.float32))
                ts.append(np.clip(np.array(labels, dtype=np.float32), 0.0, 1.0))
                ws.append(np.full(len(feats), 1.0 / len(feats), dtype=np.float32))
            report.append({"net": name, "itrs": want[1], "fixed_ms": round(fixed_ms, 3), "turns": len(trace),
                           "searched": turns, "relabelled": moved})
            log(f"{name:28s} fixed={fixed_ms:8.2f} ms turns={len(trace)} searched={turns} relabelled={moved}")
    return np.concatenate(xs), np.concatenate(ts), np.concatenate(ws), report


def init_weights(seed: int = 1) -> np.ndarray:
    """He-uniform hidden layers, small output layer, zero biases."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, fan_out, gain in ((16, 64, 2.0), (64, 64, 2.0), (64, 3, 0.1)):
        lim = math.sqrt(3.0 * gain / fan_in)
        parts.append(rng.uniform(-lim, lim, size=(fan_out, fan_in)).astype(np.float32).ravel())
        parts.append(np.zeros(fan_out, dtype=np.float32))
    w = np.concatenate(parts)
    assert w.size == hvm.POLICY_PARAMS
    return w


def evaluate(nets, weights, reps: int, log=print) -> list[dict]:
    rows = []
    for name, code in nets:
        with hvm.Runtime(device=0) as rt:
            stream = _load(rt, code)
            rt.set_policy(hvm.POLICY_FIXED)
            fixed_ms, st0 = timed_run(rt, reps, stream)
            want = _outcome(rt, st0, stream)
            rt.set_policy(hvm.POLICY_LEARNED, weights=weights)
            ms, st = timed_run(rt, reps, stream)
            if _outcome(rt, st, stream) != want:
                raise RuntimeError(f"{name}: learned schedule changed the result")
        rows.append({"net": name, "fixed_ms": round(fixed_ms, 3), "learned_ms": round(ms, 3),
                     "speedup": round(fixed_ms / ms, 3)})
        log(f"{name:28s} fixed={fixed_ms:8.2f} ms learned={ms:8.2f} ms x{fixed_ms / ms:.3f}")
    return rows


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "policy_weights.json"))
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--epochs", type=int, default=4000)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--trace-cap", type=int, default=8192)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--streams", type=int, default=0,
                    help="also train on two continuously batched streams of this many nets each")
    ap.add_argument("--labels", choices=("search", "constant"), default="search",
                    help="per-decision local search (default), or the best constant schedule per net")
    args = ap.parse_args()
    t0 = time.time()
    nets = training_nets() + (training_streams(args.streams) if args.streams else [])
    if args.labels == "search":
        x, t, sw, report = search(nets, args.reps, args.trace_cap)
    else:
        x, t, sw, report = collect(nets, args.reps, args.trace_cap)
    print(f"collected {len(x)} turns from {len(nets)} nets in {time.time() - t0:.1f} s")
    w0 = init_weights(args.seed)
    loss0, _ = hvm.policy_grad(w0, x, t, sw)
    t1 = time.time()
    w, loss = hvm.policy_train(w0, x, t, sw, epochs=args.epochs, lr=args.lr)
    print(f"trained {args.epochs} epochs in {time.time() - t1:.2f} s: loss {loss0:.5f} -> {loss:.5f}")
    rows = evaluate(nets, w, args.reps)
    out = {
        "format": "hvm_gb300 turn-scheduler MLP 16-64-64-3, packed W1 b1 W2 b2 W3 b3 (float32)",
        "params": [float(v) for v in w],
        "training": {"labels": args.labels, "nets": report, "turns": int(len(x)), "epochs": args.epochs, "lr": args.lr,
                     "loss_initial": loss0, "loss_final": loss, "seed": args.seed},
        "evaluation": rows,
    }
    with open(args.out, "w") as f:
        json.dump(out, f)
    print(f"wrote {args.out}")


def load_weights(path: str | None = None) -> np.ndarray:
    """The committed policy weights (float32, POLICY_PARAMS)."""
    with open(path or os.path.join(HERE, "policy_weights.json")) as f:
        w = np.asarray(json.load(f)["params"], dtype=np.float32)
    if w.size != hvm.POLICY_PARAMS or not np.all(np.isfinite(w)):
        raise ValueError("policy weights file is malformed")
    return w


if __name__ == "__main__":
    main()
