"""Pins the CPU oracle (oracle/hvm_oracle.c) against the reference's own C
runtime outputs (tests/golden/*.json): same normal form and same interaction
count, with one worker and with several (work stealing)."""
from __future__ import annotations

import pytest


def test_oracle_reference_programs(hvm, oracle, ref_programs):
    n = 0
    for p in ref_programs:
        if "result" not in p or p["itrs"] > 30_000_000:
            continue
        for threads in (1, 4):
            out = oracle(p["code"], threads=threads)
            assert out["itrs"] == p["itrs"], (p["name"], threads)
            assert hvm.canonical(out["result"]) == hvm.canonical(p["result"]), (p["name"], threads)
        n += 1
    assert n >= 10


@pytest.mark.parametrize("name,make", [
    ("tree_sum_d12", lambda W: W.tree_sum(12)),
    ("bitonic_sort_2p8", lambda W: W.bitonic_sort(8)),
    ("skewed_fold_2p10", lambda W: W.skewed_fold(10)),
    ("countdown_100000", lambda W: W.countdown(100000)),
])
def test_oracle_configs_small(hvm, oracle, workloads, config_goldens, name, make):
    import hashlib
    g = config_goldens[name]
    out = oracle(make(workloads), threads=2)
    assert out["itrs"] == g["itrs"]
    assert hashlib.sha256(hvm.canonical(out["result"]).encode()).hexdigest() == g["canonical_sha256"]


def test_oracle_planted_mistake_is_caught(hvm, oracle, ref_programs):
    # A wrong program (one operator changed) must not match the golden: the
    # comparison has teeth.
    p = next(x for x in ref_programs if x["name"].endswith("numerics/u24.hvm"))
    bad = p["code"].replace("[+]", "[-]", 1)
    assert bad != p["code"]
    out = oracle(bad)
    assert hvm.canonical(out["result"]) != hvm.canonical(p["result"])
