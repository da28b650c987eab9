"""The autotuner: its search space on CPU, and one small tuning run on the GPU
(every candidate must reproduce the reference's result; the winner is one of
the candidates)."""
from __future__ import annotations

import importlib

import pytest


def test_candidates_cover_the_space():
    at = importlib.import_module("lambdavm-rust_gb300.autotune")
    space = {"reg_cap_blocks": (5, 8), "graph_turns": (0, 4), "policy": ("fixed", "learned")}
    cands = at.candidates(space)
    assert len(cands) == 8
    assert {tuple(sorted(c.items())) for c in cands} == {
        tuple(sorted({"reg_cap_blocks": r, "graph_turns": g, "policy": p}.items()))
        for r in (5, 8) for g in (0, 4) for p in ("fixed", "learned")}
    # The default space (the fast-path kernel variants exist for every cap it holds).
    default = at.candidates()
    assert len(default) == 3 * 2 * 2 * 2
    assert not at.candidates({"reg_cap_blocks": (6,), "fast_calls": (1,)})


@pytest.mark.gpu
def test_tune_single_on_a_small_net(hvm, workloads, config_goldens):
    at = importlib.import_module("lambdavm-rust_gb300.autotune")
    book = hvm.book_from_text(workloads.tree_sum(12))
    space = {"reg_cap_blocks": (5, 8), "policy": ("fixed", "learned")}
    best, rows = at.tune_single(book, space=space, reps=1)
    assert best in at.candidates(space)
    assert len(rows) == 4 and all(r["ms"] > 0 for r in rows)
