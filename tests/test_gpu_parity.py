"""Parity of the sm_103a evaluator with the oracle and the reference's
goldens: bit-exact normal form (canonical tree: structure, REF names, 29-bit
numbers) and identical interaction count. All calls go through the C ABI."""
from __future__ import annotations

import hashlib
import importlib
import re
import subprocess

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rt(hvm):
    r = hvm.Runtime(device=0)
    yield r
    r.close()


def run(rt, code):
    rt.load(code)
    st = rt.run()
    return rt.result(), st


def test_reference_programs(hvm, rt, ref_programs):
    n = 0
    for p in ref_programs:
        if "result" not in p:
            continue
        res, st = run(rt, p["code"])
        assert st.itrs == p["itrs"], p["name"]
        assert hvm.canonical(res) == hvm.canonical(p["result"]), p["name"]
        n += 1
    assert n >= 12


@pytest.mark.parametrize("name", ["tree_sum_d12", "bitonic_sort_2p8", "bitonic_sort_2p12",
                                  "skewed_fold_2p10", "countdown_100000"])
def test_configs_small(hvm, rt, workloads, config_goldens, name):
    makers = {
        "tree_sum_d12": lambda: workloads.tree_sum(12),
        "bitonic_sort_2p8": lambda: workloads.bitonic_sort(8),
        "bitonic_sort_2p12": lambda: workloads.bitonic_sort(12),
        "skewed_fold_2p10": lambda: workloads.skewed_fold(10),
        "countdown_100000": lambda: workloads.countdown(100000),
    }
    res, st = run(rt, makers[name]())
    g = config_goldens[name]
    assert st.itrs == g["itrs"]
    assert hashlib.sha256(hvm.canonical(res).encode()).hexdigest() == g["canonical_sha256"]


def test_live_oracle_seeded_nets(hvm, rt, workloads, oracle):
    # Seeded nets the goldens do not hold: compared with the oracle live.
    for seed in (1, 2, 3):
        code = workloads.bitonic_sum(7, seed)
        want = oracle(code, threads=2)
        res, st = run(rt, code)
        assert st.itrs == want["itrs"]
        assert hvm.canonical(res) == hvm.canonical(want["result"])


@pytest.mark.parametrize("cfg", [dict(narrow_below=0), dict(narrow_below=1 << 30),
                                 dict(narrow_below=4096, narrow_reg_cap=5), dict(reg_cap_blocks=0, narrow_reg_cap=8)],
                         ids=["one_variant", "always_narrow", "narrow_cap5", "narrow_wider_than_wide"])
def test_kernel_variant_switching(hvm, workloads, config_goldens, cfg):
    # Turns move between the two kernel variants (different grids) at host
    # polls; the next turn is re-planned for the new grid. Every setting gives
    # the reference's interaction count and normal form.
    cases = {"tree_sum_d12": workloads.tree_sum(12), "bitonic_sort_2p12": workloads.bitonic_sort(12),
             "skewed_fold_2p10": workloads.skewed_fold(10), "countdown_100000": workloads.countdown(100000)}
    with hvm.Runtime(device=0, **cfg) as r:
        for name, code in cases.items():
            res, st = run(r, code)
            g = config_goldens[name]
            assert st.itrs == g["itrs"], name
            assert hashlib.sha256(hvm.canonical(res).encode()).hexdigest() == g["canonical_sha256"], name


@pytest.mark.parametrize("cfg", [dict(fast_calls=1), dict(fast_calls=2), dict(fast_calls=2, rule_select=0),
                                 dict(fast_calls=1, reg_cap_blocks=0), dict(rule_select=2), dict(local_nets=1),
                                 dict(local_nets=1, reg_cap_blocks=0, narrow_below=0), dict(persistent=1),
                                 dict(persistent=1, narrow_below=0), dict(persistent=1, reg_cap_blocks=0, narrow_below=0)],
                         ids=["fast_switch", "fast_switch_anni", "fast_all_lanes", "fast_uncapped", "rule_per_round",
                              "local_nets", "local_nets_uncapped", "persistent", "persistent_one_variant",
                              "persistent_uncapped"])
def test_scheduling_options(hvm, workloads, config_goldens, ref_programs, cfg):
    # CALL-time fast paths (the reference's compiled-mode short-cuts, adding
    # by hand the interactions they perform), the per-round rule selection
    # and the block-local nets (fresh words in shared memory, LEAK to HBM)
    # change how the net is reduced, never the normal form or the
    # interaction count.
    cases = {"tree_sum_d12": workloads.tree_sum(12), "bitonic_sort_2p12": workloads.bitonic_sort(12),
             "skewed_fold_2p10": workloads.skewed_fold(10), "countdown_100000": workloads.countdown(100000)}
    with hvm.Runtime(device=0, **cfg) as r:
        for name, code in cases.items():
            res, st = run(r, code)
            g = config_goldens[name]
            assert st.itrs == g["itrs"], name
            assert hashlib.sha256(hvm.canonical(res).encode()).hexdigest() == g["canonical_sha256"], name
        for prog in ref_programs:
            if "result" not in prog:
                continue
            res, st = run(r, prog["code"])
            assert st.itrs == prog["itrs"], prog["name"]
            assert hvm.canonical(res) == hvm.canonical(prog["result"]), prog["name"]


def test_persistent_launch_count(hvm, workloads, config_goldens):
    # A persistent normalisation closes its turns on the device: a handful of
    # launches for a net that runs tens of turns, the same result.
    code = workloads.bitonic_sort(12)
    with hvm.Runtime(device=0, persistent=1) as r:
        res, st = run(r, code)
        assert st.itrs == config_goldens["bitonic_sort_2p12"]["itrs"]
        assert st.turns > 8
        assert st.turn_launches <= 4
        # The learned scheduler's inference runs in the closing block as well.
        train = importlib.import_module("lambdavm-rust_gb300.train_policy")
        r.set_policy(hvm.POLICY_LEARNED, weights=train.load_weights())
        res2, st2 = run(r, code)
        assert st2.itrs == st.itrs and hvm.canonical(res2) == hvm.canonical(res)


def test_persistent_wait_limit(hvm, rt, workloads):
    # The bounded wait of persistent launches, on a word nothing writes: the
    # limit runs out, the kernel returns, and the context still runs a net.
    timed_out, ms = hvm.wait_probe(limit_ms=100)
    assert timed_out
    assert 90.0 <= ms < 5000.0
    res, st = run(rt, workloads.tree_sum(8))
    assert res == "256"


def test_repeat_runs_identical(hvm, rt, workloads):
    code = workloads.bitonic_sort(10)
    outs = {run(rt, code)[0] for _ in range(3)}
    canon = {hvm.canonical(o) for o in outs}
    assert len(canon) == 1


@pytest.mark.slow
@pytest.mark.parametrize("name", ["tree_sum_d20", "bitonic_sort_2p16", "skewed_fold_2p18"])
def test_configs_full(hvm, rt, workloads, config_goldens, name):
    makers = {
        "tree_sum_d20": lambda: workloads.tree_sum(20),
        "bitonic_sort_2p16": lambda: workloads.bitonic_sort(16),
        "skewed_fold_2p18": lambda: workloads.skewed_fold(18),
    }
    res, st = run(rt, makers[name]())
    g = config_goldens[name]
    assert st.itrs == g["itrs"]
    assert hashlib.sha256(hvm.canonical(res).encode()).hexdigest() == g["canonical_sha256"]
    if name.startswith("bitonic"):
        # size-independent property: the leaves are the sorted input keys
        got = [int(x) for x in re.findall(r"\d+", res)]
        assert got == sorted(workloads.pcg_keys(1 << 16))


def test_hvm_cu_cli(hvm, tmp_path, workloads):
    src = tmp_path / "t.hvm"
    src.write_text(workloads.tree_sum(10))
    out = subprocess.run([hvm.CLI_PATH, "run-cu", str(src)], capture_output=True, text=True, check=True).stdout
    lines = out.strip().splitlines()
    assert lines[0] == "Result: 1024"
    assert lines[1] == "- ITRS: 16374"
    assert lines[2].startswith("- LEAK: ")
    assert re.match(r"- TIME: \d+\.\d\ds", lines[3])
    assert lines[4].startswith("- MIPS: ")


def test_errors_are_reported_not_hung(hvm, workloads, ref_programs):
    # A node space too small for the net ends in an error status, not a hang:
    # examples/sum_tree builds a 2^20-leaf tree (2^21 live nodes) first.
    code = next(p["code"] for p in ref_programs if p["name"] == "examples/sum_tree/main.hvm")
    with hvm.Runtime(device=0, node_log2=19, threads_per_block=32, blocks_per_sm=1) as r:
        r.load(code)
        with pytest.raises(hvm.HvmError, match="out of node memory|ring"):
            r.run()
    # A turn budget that ends before the normal form is reported.
    with hvm.Runtime(device=0, max_turns=1) as r:
        r.load(workloads.countdown(100000))
        with pytest.raises(hvm.HvmError, match="turn budget"):
            r.run()


def test_atomic_peak_probe(hvm):
    # The atomic roofline's denominator: positive and of the right order for
    # an L2 (between 1e8 and 1e13 random 32-bit exchanges per second).
    v = hvm.atomic_peak(1 << 20)
    assert 1e8 < v < 1e13
    with pytest.raises(hvm.HvmError):
        hvm.atomic_peak(1000)  # not a power of two
