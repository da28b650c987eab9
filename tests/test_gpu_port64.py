"""The 64-bit port build (libhvm_gb300_p64.so): the same evaluator over 64-bit
ports and 128-bit node pairs, whose word indices reach 2^32 per space where
32-bit ports stop at 2^29 (the 64-bit ports the HVM2 paper proposes for larger
nets, paper/HVM2.typst:1210-1220; the reference has no such mode, so parity is
the reference's own results: the same normal forms and interaction counts as
the 32-bit runtime's goldens).

`upper_half` makes the allocator hand out words from the upper half of each
space only; with 2^32-word spaces every node and var index a run touches is
then near 2^31 or above, far past 2^29 (the words a 32-bit port can address),
so each port that points into the net carries a value above 32 bits, and any
narrowing of a port on the 64-bit path would change the result."""
from __future__ import annotations

import hashlib
import json
import os

import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch_goldens():
    with open(os.path.join(GOLDEN, "batch_mixed_4096.json")) as f:
        return json.load(f)

CASES = ("tree_sum_d12", "bitonic_sort_2p12", "skewed_fold_2p10", "countdown_100000")


def _cases(workloads):
    return {"tree_sum_d12": workloads.tree_sum(12), "bitonic_sort_2p12": workloads.bitonic_sort(12),
            "skewed_fold_2p10": workloads.skewed_fold(10), "countdown_100000": workloads.countdown(100000)}


def _run(rt, code):
    rt.load(code)
    st = rt.run()
    return rt.result(), st


@pytest.mark.parametrize("cfg", [dict(), dict(node_log2=32, vars_log2=32, upper_half=1),
                                 dict(node_log2=32, vars_log2=32, upper_half=1, persistent=1),
                                 dict(reg_cap_blocks=0, narrow_below=0)],
                         ids=["default_spaces", "upper_half_2p32", "upper_half_2p32_persistent", "uncapped"])
def test_port64_configs_match_goldens(hvm, workloads, config_goldens, ref_programs, cfg):
    with hvm.Runtime(device=0, port64=True, **cfg) as r:
        for name, code in _cases(workloads).items():
            res, st = _run(r, code)
            g = config_goldens[name]
            assert st.itrs == g["itrs"], name
            assert hashlib.sha256(hvm.canonical(res).encode()).hexdigest() == g["canonical_sha256"], name
        for prog in ref_programs:
            if "result" not in prog:
                continue
            res, st = _run(r, prog["code"])
            assert st.itrs == prog["itrs"], prog["name"]
            assert hvm.canonical(res) == hvm.canonical(prog["result"]), prog["name"]


def test_port64_high_indices_are_used(hvm, workloads):
    # With upper_half the result's vars are named by their word index: an
    # index past 2^29 cannot be held by a 32-bit port.
    with hvm.Runtime(device=0, port64=True, node_log2=32, vars_log2=32, upper_half=1) as r:
        r.load("@main = (x x)\n")  # the identity: a var in the normal form
        r.run()
        res = r.result()
    names = [tok for tok in res.replace("(", " ").replace(")", " ").split() if tok.startswith("x")]
    assert names and all(int(n[1:], 16) >= 1 << 30 for n in names), res


@pytest.mark.parametrize("cfg", [dict(), dict(node_log2=32, vars_log2=32, upper_half=1)],
                         ids=["default_spaces", "upper_half_2p32"])
def test_port64_batch_matches_goldens(hvm, batch_goldens, workloads, cfg):
    # The first 256 nets of the mixed batch, run together.
    nets = workloads.mixed_batch(4096)[:256]
    with hvm.Runtime(device=0, port64=True, **cfg) as r:
        r.load_batch([code for code, _ in nets])
        st = r.run_batch()
        got = [r.batch_result(i) for i in range(len(nets))]
    bad = [(i, got[i], batch_goldens["nets"][i]["result"]) for i in range(len(nets))
           if got[i] != str(batch_goldens["nets"][i]["result"])]
    assert not bad, bad[:8]
    assert st.itrs == sum(batch_goldens["nets"][i]["itrs"] for i in range(len(nets)))


@pytest.mark.slow
@pytest.mark.parametrize("name", ["tree_sum_d20", "bitonic_sort_2p16", "skewed_fold_2p18"])
def test_port64_configs_full(hvm, workloads, config_goldens, name):
    makers = {"tree_sum_d20": lambda: workloads.tree_sum(20), "bitonic_sort_2p16": lambda: workloads.bitonic_sort(16),
              "skewed_fold_2p18": lambda: workloads.skewed_fold(18)}
    with hvm.Runtime(device=0, port64=True, node_log2=32, vars_log2=32) as r:
        res, st = _run(r, makers[name]())
    g = config_goldens[name]
    assert st.itrs == g["itrs"]
    assert hashlib.sha256(hvm.canonical(res).encode()).hexdigest() == g["canonical_sha256"]


def test_port64_serving_scaled_pool(hvm, workloads):
    # Serving at the stated scale: requests drawn from the serving pool (nets
    # up to 2^22 nodes) arrive as a Poisson process and run in a 64 GB arena
    # (2^31 node words of 16 B, 2^32 var words of 8 B); every response and the
    # interaction total match the reference C runtime's per-template results.
    with open(os.path.join(GOLDEN, "serving_pool.json")) as f:
        gold = json.load(f)
    books = [hvm.book_from_text(code) for code, _ in workloads.serving_pool(gold["count"])]
    arrivals, tmpl = workloads.serving_requests(64, 1e3, pool=gold["count"])
    with hvm.Runtime(device=0, port64=True, node_log2=31, vars_log2=32) as r:
        r.load_batch(books)
        r.set_requests(tmpl)
        st, done, res = r.run_stream(arrival_s=arrivals, max_inflight=512, live_frac=0.5)
    assert all(d >= a for d, a in zip(done, arrivals))
    for p, t in zip(res, tmpl):
        assert int(p) & 7 == 3 and (int(p) >> 8) == int(gold["nets"][t]["result"]), t
    assert st.itrs == sum(gold["nets"][t]["itrs"] for t in tmpl)
