#!/usr/bin/env python3
"""Benchmark of the GB300 HVM2 evaluator.

One step = one full evaluation of the benchmark net: clear the net, boot
`@main ~ ROOT`, normalise, and run the readback expansion. The default
workload is the single-net bitonic sort of 2^16 PCG32 u24 keys (the sorted
tree is the normal form). Every step's interaction count is checked against
the golden count of the reference's C runtime, and the first step's normal
form against its golden SHA-256.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
  python bench.py --impl reference ...   # the CPU evaluator on the host cores

Prints one JSON line (rank 0). `value` is interactions/s with the book
resident in HBM; `e2e` is the same metric through the C-ABI calls a user
makes (book upload from pinned host memory, evaluation, result readback)
with the copies inside the timed region. Under torchrun each rank runs its
own replica (one net per GPU: the evaluator does not shard a single net).
"""
from __future__ import annotations

import argparse
import ctypes
import hashlib
import importlib
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "interactions/s on 1 GB300, learned+batched vs plain kernel, bit-exact normal form"
UNIT = "interactions/s"
GOLDEN = os.path.join(ROOT, "tests", "golden", "configs.json")
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC = os.path.join(ROOT, "profiles", "turn_kernel_bitonic_2p14.md")
ORACLE = os.path.join(ROOT, "oracle", "_build", "hvm_oracle")

BATCH_GOLDEN = os.path.join(ROOT, "tests", "golden", "batch_mixed_4096.json")

WORKLOADS = {
    # name: (golden key, generator, description)
    "bitonic_sort_2p16": ("bitonic_sort_2p16", lambda W: W.bitonic_sort(16),
                          "bitonic sort of 2^16 PCG32 u24 keys, single net, sorted tree as normal form"),
    "tree_sum_d20": ("tree_sum_d20", lambda W: W.tree_sum(20), "recursive tree sum d=20, single net"),
    "skewed_fold_2p18": ("skewed_fold_2p18", lambda W: W.skewed_fold(18),
                         "fold over 2^18 geometric-length countdowns, single net"),
    "batch_mixed_4096": (None, None, "4096 independent nets (1/3 tree sums d 8..18, 1/3 bitonic sorts of 2^6..2^12 "
                                     "keys then summed, 1/3 countdowns 10..1e5), continuous batching"),
    "serving": (None, None, "Poisson arrivals of nets drawn from the 4096-net mixed pool, continuous batching"),
    "compiled_calls": (None, None, "standalone `hvm gen-cu --compiled` programs against `hvm gen-cu` ones "
                                   "(bitonic 2^16, tree sum d=20, skewed fold 2^18, countdown 1e5)"),
}

# Continuous-batching settings for the mixed batch (admission cap and live-memory
# limit keep the concurrent nets' memory within the 2^29-word spaces).
BATCH_INFLIGHT = 512
BATCH_LIVE_FRAC = 0.25


def numb_u24(port: int) -> int | None:
    return ((int(port) >> 3) >> 5) if int(port) & 7 == 3 else None


def batch_check(res, gold_nets) -> bool:
    return all(numb_u24(p) == int(g["result"]) for p, g in zip(res, gold_nets))


def learned_weights():
    return importlib.import_module("lambdavm-rust_gb300.train_policy").load_weights()


def set_policy(hvm, rt, policy: str) -> None:
    if policy == "learned":
        rt.set_policy(hvm.POLICY_LEARNED, weights=learned_weights())
    else:
        rt.set_policy(hvm.POLICY_FIXED)


def bench_batch(hvm, W, args, plain_sample: int = 128, policy: str = "fixed", cfg: dict | None = None) -> dict:
    """The 4096-net mixed batch through continuous batching, and the
    plain path (one net per evaluation) on an evenly spaced sample of it."""
    gold = json.load(open(BATCH_GOLDEN))
    nets = W.mixed_batch(gold["count"])
    books = [hvm.book_from_text(code) for code, _ in nets]
    rt = hvm.Runtime(device=0, **(cfg or {}))
    set_policy(hvm, rt, policy)
    rt.load_batch(books)
    for _ in range(max(1, args.warmup // 3)):
        st, done, res = rt.run_stream(max_inflight=BATCH_INFLIGHT, live_frac=BATCH_LIVE_FRAC)
    secs, ok = [], True
    for _ in range(max(1, args.steps // 10)):
        t0 = time.perf_counter()
        st, done, res = rt.run_stream(max_inflight=BATCH_INFLIGHT, live_frac=BATCH_LIVE_FRAC)
        secs.append(time.perf_counter() - t0)
        ok = ok and st.itrs == gold["total_itrs"] and batch_check(res, gold["nets"])
    batched = gold["total_itrs"] / statistics.median(secs)
    out = {"nets": gold["count"], "itrs": gold["total_itrs"], "value": batched, "unit": UNIT,
           "seconds": statistics.median(secs), "p50_done_s": float(sorted(done)[len(done) // 2]),
           "max_done_s": float(done.max()), "max_inflight": BATCH_INFLIGHT, "live_frac": BATCH_LIVE_FRAC,
           "parity": bool(ok), "policy": policy, "config": cfg or {}}
    if not plain_sample:
        rt.close()
        return out
    # plain: nets one at a time through the single-net path
    step = max(1, len(books) // plain_sample)
    t0 = time.perf_counter()
    p_itrs = 0
    for k in range(0, len(books), step):
        rt.load(books[k])
        s = rt.run()
        p_itrs += s.itrs
        ok = ok and s.itrs == gold["nets"][k]["itrs"]
    plain = p_itrs / (time.perf_counter() - t0)
    rt.close()
    out["plain_kernel"] = {"value": plain, "sample_nets": len(range(0, len(books), step)),
                           "note": "same nets, one per evaluation (single-net path)"}
    out["batched_over_plain"] = batched / plain
    out["parity"] = bool(ok)
    return out


def bench_scheduler(hvm, W, reps: int = 5) -> dict:
    """The skewed fold over 2^18 countdowns under the fixed and the
    learned turn policy (median wall time of `reps` evaluations each, book
    resident; every run checked against the reference's interaction count and
    normal form)."""
    golden = json.load(open(GOLDEN))["skewed_fold_2p18"]
    book = hvm.book_from_text(W.skewed_fold(18))
    out = {"workload": "fold over 2^18 geometric-length countdowns (p = 1/64, cap 2^16), single net",
           "itrs": golden["itrs"]}
    for policy in ("fixed", "learned"):
        with hvm.Runtime(device=0) as rt:
            set_policy(hvm, rt, policy)
            rt.load(book)
            st = rt.run()
            ok = st.itrs == golden["itrs"] and \
                hashlib.sha256(hvm.canonical(rt.result()).encode()).hexdigest() == golden["canonical_sha256"]
            ms = []
            for _ in range(reps):
                t0 = time.perf_counter()
                st = rt.run()
                ms.append((time.perf_counter() - t0) * 1e3)
                ok = ok and st.itrs == golden["itrs"]
            med = statistics.median(ms)
            out[policy] = {"value": golden["itrs"] / med * 1e3, "unit": UNIT, "ms": med, "turns": st.turns,
                           "parity": bool(ok)}
    out["learned_over_fixed"] = out["learned"]["value"] / out["fixed"]["value"]
    return out


def bench_compiled_calls(hvm, W, reps: int = 3) -> dict:
    """Compiled calls against the table-driven CALL: for each workload the
    standalone programs of `hvm gen-cu --compiled` and `hvm gen-cu`, built
    with nvcc for sm_103a, each run `reps` times as its own process with
    kernels loaded eagerly (so the printed MIPS covers the evaluation only:
    boot, turns and readback). Every run is checked against the reference's
    interaction count and normal form."""
    from concurrent.futures import ThreadPoolExecutor
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    golden = json.load(open(GOLDEN))
    cases = [("bitonic_sort_2p16", W.bitonic_sort(16)), ("tree_sum_d20", W.tree_sum(20)),
             ("skewed_fold_2p18", W.skewed_fold(18)), ("countdown_100000", W.countdown(100000))]
    tmp = tempfile.mkdtemp(prefix="hvm_cc_")
    jobs = []
    for name, code in cases:
        src = os.path.join(tmp, name + ".hvm")
        open(src, "w").write(code)
        for arm in ("interpreted", "compiled"):
            cmd = [hvm.CLI_PATH, "gen-cu"] + (["--compiled"] if arm == "compiled" else []) + [src]
            cu = os.path.join(tmp, f"{name}_{arm}.cu")
            open(cu, "w").write(subprocess.run(cmd, capture_output=True, text=True, check=True).stdout)
            jobs.append((name, arm, cu, cu[:-3]))

    def build(job):
        _, _, cu, exe = job
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", cu, "-o", exe],
                       check=True, capture_output=True, timeout=900)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(build, jobs))
    build_s = time.perf_counter() - t0
    env = dict(os.environ, CUDA_MODULE_LOADING="EAGER")
    out = {}
    for name, arm, _, exe in jobs:
        g = golden[name]
        mips, ok = [], True
        for _ in range(reps):
            txt = subprocess.run([exe], capture_output=True, text=True, check=True, env=env, timeout=600).stdout
            res = re.search(r"^Result: (.*)$", txt, re.M).group(1)
            itrs = int(re.search(r"^- ITRS: (\d+)$", txt, re.M).group(1))
            mips.append(float(re.search(r"^- MIPS: ([0-9.]+)$", txt, re.M).group(1)))
            ok = ok and itrs == g["itrs"] and \
                hashlib.sha256(hvm.canonical(res).encode()).hexdigest() == g["canonical_sha256"]
        row = out.setdefault(name, {"itrs": g["itrs"]})
        row[arm + "_itrs_per_s"] = statistics.median(mips) * 1e6
        row[arm + "_parity"] = bool(ok)
    for row in out.values():
        row["compiled_over_interpreted"] = row["compiled_itrs_per_s"] / row["interpreted_itrs_per_s"]
    return {"workloads": out, "reps": reps, "nvcc_build_s": build_s,
            "note": "median of reps; each run is one process (runtime creation excluded from its timing)"}


def bench_serving(hvm, W, rates=(1e2, 1e3, 1e4, 1e5), seconds: float = 2.0, max_requests: int = 100_000) -> dict:
    """Serving: Poisson arrivals at each rate for about `seconds` of arrivals
    (at most `max_requests`), nets drawn from the 4096-net pool; latency =
    completion - arrival on the host clock; every response checked against
    the reference's result for its net."""
    gold = json.load(open(BATCH_GOLDEN))
    nets = W.mixed_batch(gold["count"])
    books = [hvm.book_from_text(code) for code, _ in nets]
    rt = hvm.Runtime(device=0)
    out = []
    for rate in rates:
        n = int(min(max_requests, max(50, rate * seconds)))
        arrivals, tmpl = W.serving_requests(n, rate)
        rt.load_batch(books)
        rt.set_requests(tmpl)
        t0 = time.perf_counter()
        st, done, res = rt.run_stream(arrival_s=arrivals, max_inflight=BATCH_INFLIGHT, live_frac=BATCH_LIVE_FRAC)
        wall = time.perf_counter() - t0
        lat = sorted(float(d - a) for d, a in zip(done, arrivals))
        ok = all(numb_u24(p) == int(gold["nets"][t]["result"]) for p, t in zip(res, tmpl))
        itrs_expected = sum(gold["nets"][t]["itrs"] for t in tmpl)
        out.append({"rate_per_s": rate, "requests": n, "wall_s": wall, "itrs": st.itrs,
                    "itrs_per_s": st.itrs / wall, "p50_latency_s": lat[len(lat) // 2],
                    "p99_latency_s": lat[min(len(lat) - 1, int(len(lat) * 0.99))],
                    "parity": bool(ok and st.itrs == itrs_expected)})
    rt.close()
    return {"rates": out}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """torch.distributed around the replicas (barrier, max over ranks)."""

    def __init__(self, ws: int, rank: int, local: int, use_cuda: bool):
        self.ws, self.rank, self.local = ws, rank, local
        self.torch = None
        if ws > 1:
            import torch
            import torch.distributed as td
            self.torch = torch
            backend = "nccl" if use_cuda else "gloo"
            if use_cuda:
                torch.cuda.set_device(local)
            td.init_process_group(backend=backend)
            self.td = td
            self.dev = torch.device("cuda", local) if use_cuda else torch.device("cpu")

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.ws == 1:
            return x
        t = self.torch.tensor([x], dtype=self.torch.float64, device=self.dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self.ws == 1:
            return x
        t = self.torch.tensor([x], dtype=self.torch.float64, device=self.dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        rows = [l.split(",") for l in open(self.path).read().splitlines() if l.strip()]
        os.unlink(self.path)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
            except ValueError:
                continue
            for name, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def read_traffic_per_itr() -> float | None:
    try:
        m = re.search(r"traffic_bytes_per_interaction:\s*([0-9.]+)", open(TRAFFIC).read())
        return float(m.group(1)) if m else None
    except OSError:
        return None


def run_oracle(book, threads: int) -> tuple[int, float, str]:
    with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as f:
        book.tofile(f.name)
        path = f.name
    try:
        out = subprocess.run([ORACLE, "-t", str(threads), "-n", path], capture_output=True, text=True,
                             check=True).stdout
    finally:
        os.unlink(path)
    itrs = int(re.search(r"^- ITRS: (\d+)$", out, re.M).group(1))
    ns = int(re.search(r"^- NORM_NS: (\d+)$", out, re.M).group(1))
    res = re.search(r"^Result: (.*)$", out, re.M).group(1)
    return itrs, ns / 1e9, res


def ensure_built():
    pkg = importlib.import_module("lambdavm-rust_gb300")
    if not os.path.exists(pkg.LIB_PATH) or not os.path.exists(ORACLE):
        importlib.import_module("__graft_entry__").build()
    return pkg


def bench_reference(args, book, golden, desc, ws, rank):
    """The reference's CPU evaluator (its work-stealing pthreads algorithm,
    restated in oracle/hvm_oracle.c) on all host cores, same workload."""
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    times = []
    for i in range(args.warmup + args.steps):
        itrs, secs, _ = run_oracle(book, threads)
        if itrs != golden["itrs"]:
            raise SystemExit(f"oracle interaction count {itrs} != golden {golden['itrs']}")
        if i >= args.warmup:
            times.append(secs)
    value = golden["itrs"] / statistics.mean(times)
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(times) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": desc, "itrs_per_step": golden["itrs"]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"full workload ({golden['itrs']} interactions) per step, {threads} worker threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def bench_gpu(args, hvm, book, golden, desc, ws, rank, local, dist):
    import torch
    torch.cuda.set_device(local)
    rt = hvm.Runtime(device=local)

    # Warm-up, with a full parity check of the first step.
    rt.load(book)
    for i in range(args.warmup):
        st = rt.run()
        if st.itrs != golden["itrs"]:
            raise SystemExit(f"interaction count {st.itrs} != golden {golden['itrs']}")
        if i == 0:
            canon = hvm.canonical(rt.result())
            if hashlib.sha256(canon.encode()).hexdigest() != golden["canonical_sha256"]:
                raise SystemExit("normal form differs from the golden")

    # value: book resident in HBM; each step clears the 6 GB net (which also
    # flushes L2), boots, normalises and expands.
    rt.reset_counters()
    sampler = ClockSampler(local)
    sampler.start()
    dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    itrs_total = 0
    for _ in range(args.steps):
        st = rt.run()
        itrs_total += st.itrs
        if st.itrs != golden["itrs"]:
            raise SystemExit(f"interaction count {st.itrs} != golden {golden['itrs']}")
    ev1.record()
    torch.cuda.synchronize()
    dist.barrier()
    clocks = sampler.stop()
    secs = ev0.elapsed_time(ev1) / 1e3
    counters = st  # the last step's stats carry the counters accumulated since reset_counters
    kernel_s = counters.kernel_ms / 1e3
    turns_effective = counters.turns * args.steps  # turns per evaluation x steps
    launches = counters.launches

    # e2e: the C-ABI calls a user makes, with the book copied from pinned host
    # memory and the result read back to the host inside the timed region.
    pinned = torch.from_numpy(book.view("int32")).pin_memory()
    rt.reset_counters()
    dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        L = hvm.lib()
        rc = L.hvm_gb300_load_book(rt._h, ctypes.cast(pinned.data_ptr(), ctypes.POINTER(ctypes.c_uint32)),
                                   book.size)
        if rc:
            raise SystemExit(L.hvm_gb300_error(rt._h).decode())
        st_e = rt.run()
        res = rt.result()
        if st_e.itrs != golden["itrs"] or not res:
            raise SystemExit("e2e step failed its check")
    e1.record()
    torch.cuda.synchronize()
    dist.barrier()
    e2e_secs = e0.elapsed_time(e1) / 1e3
    h2d = st_e.h2d_bytes // args.steps
    d2h = st_e.d2h_bytes // args.steps

    secs_max = dist.max(secs)
    e2e_max = dist.max(e2e_secs)
    value = dist.sum(itrs_total) / secs_max
    e2e_value = dist.sum(golden["itrs"] * args.steps) / e2e_max
    rt.close()
    if rank != 0:
        return None

    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    peak = peaks.get("hbm_gbs")
    peak_note = "measured" if peak else "fallback"
    if not peak:
        peak = 6800.0
    bpi = golden["algorithmic_bytes"] / golden["itrs"]
    achieved = bpi * itrs_total / kernel_s / 1e9 if kernel_s > 0 else None
    tpi = read_traffic_per_itr()
    itrs_per_launch = itrs_total / max(1, turns_effective)
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak if achieved else None,
        "traffic": tpi * itrs_per_launch if tpi else None,
        "peak_source": peak_note,
        "kernel": "turn_kernel",
        "algorithmic_bytes_per_interaction": bpi,
        "interactions_per_launch": itrs_per_launch,
        "avg_launch_ms": counters.kernel_ms / max(1, turns_effective),
    }
    # Second roofline: the model's atomic operations (node takes + var
    # exchanges, counted by the oracle) against the measured atomicExch
    # throughput at random addresses of a 64 MB region (L2-resident) and of
    # a 2 GB one (the var space's size).
    roofline_atomic = None
    if golden.get("algorithmic_atomics"):
        api = golden["algorithmic_atomics"] / golden["itrs"]
        peak_l2 = hvm.atomic_peak(1 << 24, local) / 1e9
        peak_far = hvm.atomic_peak(1 << 29, local) / 1e9
        ach = api * itrs_total / kernel_s / 1e9 if kernel_s > 0 else None
        roofline_atomic = {"bound": "l2_atomics", "achieved": ach, "peak": peak_l2, "unit": "Gatomic/s",
                           "frac": ach / peak_l2 if ach else None, "peak_2gb_region": peak_far,
                           "frac_of_2gb_region": ach / peak_far if ach else None,
                           "atomics_per_interaction": api, "peak_source": "measured by hvm_gb300_atomic_peak"}
    # CPU baseline: the oracle port on this host's cores, one full evaluation.
    threads = os.cpu_count() or 1
    c_itrs, c_secs, _ = run_oracle(book, threads)
    cpu = {"value": c_itrs / c_secs, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"one full evaluation of the same workload ({c_itrs} interactions), {threads} worker threads"}
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs_max / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": desc, "itrs_per_step": golden["itrs"], "policy": "fixed",
                   "threads": counters.threads, "parallelism": f"replicas x{ws}",
                   "l2": "each step clears the 6 GB node/var space (> L2) before evaluating",
                   "parity": "interaction count checked every step; normal form SHA-256 checked"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": roofline,
        "roofline_atomic": roofline_atomic,
        "cpu_baseline": cpu,
        "clocks": clocks,
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="bitonic_sort_2p16")
    ap.add_argument("--no-batch", action="store_true", help="skip the 4096-net batch report of the default line")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    hvm = ensure_built()
    W = importlib.import_module("lambdavm-rust_gb300.workloads")
    key, make, desc = WORKLOADS[args.workload]
    if args.workload == "compiled_calls":
        if args.impl == "reference" or rank != 0:
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the CPU arm runs the single-net workloads"}))
            return
        cc = bench_compiled_calls(hvm, W)
        b = cc["workloads"]["bitonic_sort_2p16"]
        line = {"metric": METRIC, "value": b["compiled_itrs_per_s"], "unit": UNIT, "n_gpus": 1, "steps": cc["reps"],
                "warmup": 0, "ms_per_step": b["itrs"] / b["compiled_itrs_per_s"] * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
                "config": {"workload": desc, **cc}}
        print(json.dumps(line), flush=True)
        return
    if args.workload in ("batch_mixed_4096", "serving"):
        if args.impl == "reference" or rank != 0:
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the CPU arm runs the single-net workloads"}))
            return
        import torch
        torch.cuda.set_device(local)
        if args.workload == "batch_mixed_4096":
            # Autotune on the batch itself (one timed run per candidate after a
            # warm-up run), then measure the whole batch with the winner.
            at = importlib.import_module("lambdavm-rust_gb300.autotune")
            gold = json.load(open(BATCH_GOLDEN))
            sample = [hvm.book_from_text(code) for code, _ in W.mixed_batch(gold["count"])]
            space = {"reg_cap_blocks": (5, 8), "graph_turns": (0, 4), "policy": ("fixed", "learned")}
            best, rows = at.tune_batch(sample, BATCH_INFLIGHT, BATCH_LIVE_FRAC, space=space)
            best = dict(best)
            policy = best.pop("policy")
            b = bench_batch(hvm, W, args, policy=policy, cfg=best)
            b["autotune"] = {"sample_nets": len(sample), "space": space,
                             "rows": [{**r["candidate"], "seconds": r["seconds"]} for r in rows]}
            line = {"metric": METRIC, "value": b["value"], "unit": UNIT, "n_gpus": 1, "steps": max(1, args.steps // 10),
                    "warmup": max(1, args.warmup // 3), "ms_per_step": b["seconds"] * 1e3, "higher_is_better": True,
                    "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
                    "config": {"workload": desc, **{k: v for k, v in b.items() if k not in ("value", "unit")}}}
        else:
            sv = bench_serving(hvm, W)
            best = max(r["itrs_per_s"] for r in sv["rates"])
            line = {"metric": METRIC, "value": best, "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 0,
                    "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                    "dtype": "u32", "data": "synthetic", "config": {"workload": desc, **sv}}
        print(json.dumps(line), flush=True)
        return
    golden = json.load(open(GOLDEN))[key]
    book = hvm.book_from_text(make(W))
    if args.impl == "reference":
        line = bench_reference(args, book, golden, desc, ws, rank)
        if line:
            print(json.dumps(line), flush=True)
        return
    dist = Dist(ws, rank, local, use_cuda=True)
    try:
        line = bench_gpu(args, hvm, book, golden, desc, ws, rank, local, dist)
        if line is not None and not args.no_batch:
            line["batched"] = bench_batch(hvm, W, args)
            line["batched_learned"] = bench_batch(hvm, W, args, plain_sample=0, policy="learned")
            line["scheduler"] = bench_scheduler(hvm, W)
    finally:
        dist.close()
    if line:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
