"""Batched evaluation: many independent nets in the same launches. Each net's
normal form must equal the reference's, and the batch's interaction count
must equal the sum of the nets' counts under the reference."""
from __future__ import annotations

import json
import os

import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch_golden():
    with open(os.path.join(GOLDEN, "batch_mixed_4096.json")) as f:
        return json.load(f)


def numb_value(port: int) -> int:
    assert port & 7 == 3, f"not a number: {port:#x}"
    return (port >> 3) >> 5  # u24 payload


def check_roots(roots, nets):
    for k, (p, g) in enumerate(zip(roots, nets)):
        assert numb_value(int(p)) == int(g["result"]), (k, g)


def test_batch_prefix(hvm, workloads, batch_golden):
    n = 96
    nets = workloads.mixed_batch(4096)[:n]
    gold = batch_golden["nets"][:n]
    with hvm.Runtime(device=0) as rt:
        rt.load_batch([code for code, _ in nets])
        for _ in range(2):
            st = rt.run_batch()
            assert st.itrs == sum(g["itrs"] for g in gold)
            check_roots(rt.batch_roots(), gold)
        assert hvm.canonical(rt.batch_result(5)) == hvm.canonical(gold[5]["result"])


def test_batch_of_reference_programs(hvm, ref_programs):
    # Non-numeric normal forms and the readback expansion (which re-normalises
    # REFs and adds interactions) per net of a batch.
    progs = [p for p in ref_programs if "result" in p and p["itrs"] < 200_000]
    with hvm.Runtime(device=0) as rt:
        rt.load_batch([p["code"] for p in progs])
        st = rt.run_batch()
        assert st.itrs == sum(p["itrs"] for p in progs)
        for k, p in enumerate(progs):
            assert hvm.canonical(rt.batch_result(k)) == hvm.canonical(p["result"]), p["name"]


def test_stream_prefix_matches_goldens(hvm, workloads, batch_golden):
    # Continuous batching: at most 16 nets in flight, the rest admitted as
    # others complete; every result and the total count still match.
    n = 96
    nets = workloads.mixed_batch(4096)[:n]
    gold = batch_golden["nets"][:n]
    with hvm.Runtime(device=0) as rt:
        rt.load_batch([code for code, _ in nets])
        st, done, res = rt.run_stream(max_inflight=16)
        assert st.itrs == sum(g["itrs"] for g in gold)
        check_roots(res, gold)
        assert (done > 0).all()


def test_stream_alone_and_in_the_mix(hvm, workloads, batch_golden):
    # A net's result is the same alone and admitted among others while they run.
    nets = workloads.mixed_batch(4096)[:24]
    gold = batch_golden["nets"][:24]
    with hvm.Runtime(device=0) as rt:
        for k in (1, 2, 4):
            rt.load(nets[k][0])
            st = rt.run()
            assert st.itrs == gold[k]["itrs"]
            assert hvm.canonical(rt.result()) == hvm.canonical(gold[k]["result"])
        rt.load_batch([code for code, _ in nets])
        arrivals = [0.0] * 8 + [0.002 * i for i in range(16)]  # late arrivals join running nets
        st, done, res = rt.run_stream(arrival_s=arrivals, max_inflight=12)
        check_roots(res, gold)
        assert st.itrs == sum(g["itrs"] for g in gold)


@pytest.mark.slow
def test_batch_4096(hvm, workloads, batch_golden):
    # All 4096 nets through the stream, 1024 in flight (the bench runs 512).
    # At 1536 in flight the live node set peaks near a third of the 2^29-word
    # space and the lanes' partly used pages approach the whole page pool:
    # one run in about 17 ran out of pages there.
    nets = workloads.mixed_batch(4096)
    with hvm.Runtime(device=0) as rt:
        rt.load_batch([code for code, _ in nets])
        st, done, res = rt.run_stream(max_inflight=1024, live_frac=0.25)
        assert st.itrs == batch_golden["total_itrs"]
        check_roots(res, batch_golden["nets"])


def test_serving_requests_match_goldens(hvm, workloads, batch_golden):
    # Requests drawn from a pool of nets arrive as a Poisson process while
    # others run; each response equals the reference's result for its net.
    pool = 64
    nets = workloads.mixed_batch(4096)[:pool]
    arrivals, tmpl = workloads.serving_requests(200, 5000.0, pool=pool)
    with hvm.Runtime(device=0) as rt:
        rt.load_batch([code for code, _ in nets])
        rt.set_requests(tmpl)
        st, done, res = rt.run_stream(arrival_s=arrivals, max_inflight=64)
        gold = batch_golden["nets"]
        assert st.itrs == sum(gold[t]["itrs"] for t in tmpl)
        for r, (p, t) in enumerate(zip(res, tmpl)):
            assert numb_value(int(p)) == int(gold[t]["result"]), (r, t)
        assert (done >= arrivals).all()
