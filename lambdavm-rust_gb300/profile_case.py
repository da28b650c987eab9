"""Runs one benchmark net on the GPU with a small net memory, for profilers.

ncu captures replay each kernel many times and save/restore device memory
between passes, so a profiling run should hold little memory and launch few
kernels: this evaluates one workload once (or a few times) with node/var
spaces of 2^k words and prints the interaction count, turns and time.

  python lambdavm-rust_gb300/profile_case.py --workload bitonic --log2n 14 --space-log2 26
"""
from __future__ import annotations

import argparse
import importlib
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", choices=["bitonic", "tree_sum", "skewed"], default="bitonic")
    ap.add_argument("--log2n", type=int, default=14, help="keys (bitonic), depth (tree_sum), elements (skewed)")
    ap.add_argument("--space-log2", type=int, default=26, help="node and var space: 2^k words each")
    ap.add_argument("--ring-log2", type=int, default=24)
    ap.add_argument("--runs", type=int, default=1)
    args = ap.parse_args()
    hvm = importlib.import_module("lambdavm-rust_gb300")
    W = importlib.import_module("lambdavm-rust_gb300.workloads")
    make = {"bitonic": W.bitonic_sort, "tree_sum": W.tree_sum, "skewed": W.skewed_fold}[args.workload]
    with hvm.Runtime(device=0, node_log2=args.space_log2, vars_log2=args.space_log2,
                     ring_log2=args.ring_log2) as rt:
        rt.load(make(args.log2n))
        for _ in range(args.runs):
            st = rt.run()
            print(f"itrs {st.itrs} turns {st.turns} ms {st.seconds * 1e3:.3f} kernel_ms {st.kernel_ms:.3f}", flush=True)


if __name__ == "__main__":
    main()
