"""Pins the CPU oracle (oracle/hvm_oracle.c) against the reference's own C
runtime outputs (tests/golden/*.json): same normal form and same interaction
count, with one worker and with several (work stealing)."""
from __future__ import annotations

import os
import re
import subprocess
import tempfile

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


REF_BIN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "oracle", "_ref", "hvm_ref")


def _run_reference_runtime(hvm, code: str) -> dict:
    buf = hvm.book_from_text(code)
    with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as f:
        buf.tofile(f.name)
        path = f.name
    try:
        r = subprocess.run([REF_BIN, path], capture_output=True, text=True, timeout=600)
    finally:
        os.unlink(path)
    assert r.returncode == 0, r.stderr
    return {"result": re.search(r"^Result: (.*)$", r.stdout, re.M).group(1),
            "itrs": int(re.search(r"^- ITRS: (\d+)$", r.stdout, re.M).group(1))}


@pytest.mark.skipif(not os.path.exists(REF_BIN),
                    reason="the reference's C runtime is built only where its sources are")
@pytest.mark.parametrize("make", [
    lambda W: W.bitonic_sum(6, 11), lambda W: W.bitonic_sum(7, 12), lambda W: W.bitonic_sum(8, 13),
    lambda W: W.bitonic_sort(7, seed=99), lambda W: W.skewed_fold(9, seed=7), lambda W: W.skewed_fold(8, seed=8),
    lambda W: W.tree_sum(9), lambda W: W.countdown(777),
], ids=["bsum6_s11", "bsum7_s12", "bsum8_s13", "bitonic7_s99", "skewed9_s7", "skewed8_s8", "tree9", "count777"])
def test_oracle_matches_reference_runtime_live(hvm, oracle, workloads, make):
    # Seeded nets that no golden holds: the restatement against the
    # reference's own C runtime, run here on the same buffers.
    code = make(workloads)
    want = _run_reference_runtime(hvm, code)
    for threads in (1, 3):
        got = oracle(code, threads=threads)
        assert got["itrs"] == want["itrs"], threads
        assert hvm.canonical(got["result"]) == hvm.canonical(want["result"]), threads


# The reference sources as staged by `make -C oracle stage` (or $REF_SRC).
REF_SRC = os.environ.get("REF_SRC", os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "src"))


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_SRC, "hvm.c")),
                    reason="the reference's C sources were not staged (make -C oracle stage)")
def test_gen_c_compiled_mode_matches_run_c(hvm, workloads, ref_programs, config_goldens):
    # The reference's compiled C mode (`hvm gen-c`: per-def C functions with
    # the SWITCH / OPER / COPY / ANNI / VOID fast paths, restated by
    # oracle/gen_c.py and spliced into the reference's own hvm.c/run.c) gives
    # the same normal forms and the same interaction counts as `hvm run-c`,
    # with one worker and with four: each fast path counts exactly the
    # interactions it short-cuts.
    import hashlib
    import importlib.util
    from concurrent.futures import ThreadPoolExecutor
    spec = importlib.util.spec_from_file_location(
        "gen_c", os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "oracle", "gen_c.py"))
    gen_c = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen_c)
    jobs = []
    for p in ref_programs:
        if "result" in p:
            jobs.append((re.sub(r"\W", "_", p["name"]), p["code"], p["itrs"], lambda r, p=p: hvm.canonical(r) ==
                         hvm.canonical(p["result"])))
    makers = {"tree_sum_d12": workloads.tree_sum(12), "bitonic_sort_2p8": workloads.bitonic_sort(8),
              "skewed_fold_2p10": workloads.skewed_fold(10), "countdown_100000": workloads.countdown(100000)}
    for name, code in makers.items():
        g = config_goldens[name]
        jobs.append((name, code, g["itrs"], lambda r, g=g: hashlib.sha256(hvm.canonical(r).encode()).hexdigest() ==
                     g["canonical_sha256"]))

    def check(job):
        name, code, itrs, same = job
        words = hvm.book_from_text(code)
        return [(name, t, out["itrs"] == itrs, same(out["result"]))
                for t in (0, 2) for out in [gen_c.build_and_run(words, name, tpc_l2=t)]]

    with ThreadPoolExecutor(max_workers=8) as ex:
        rows = [r for rs in ex.map(check, jobs) for r in rs]
    assert len(rows) >= 30
    for name, t, itrs_ok, nf_ok in rows:
        assert itrs_ok and nf_ok, (name, t)


def test_oracle_matches_serving_pool_goldens(hvm, oracle, workloads):
    # The serving pool's fixture came from the reference C runtime; the
    # oracle restatement reproduces every template it can finish in seconds
    # (72 of the 96, about 15 M interactions together).
    import json
    import os
    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, "serving_pool.json")) as f:
        gold = json.load(f)
    nets = workloads.serving_pool(gold["count"])
    checked = 0
    for (code, info), g in zip(nets, gold["nets"]):
        if g["itrs"] >= 2_000_000:
            continue
        out = oracle(code, threads=2)
        assert out["itrs"] == g["itrs"], info
        assert out["result"] == g["result"], info
        checked += 1
    assert checked >= 64
