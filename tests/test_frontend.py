"""Front-end (parser, builder, serializer) against the reference's layout
rules (src/ast.rs:432-634, src/hvm.rs:957-1003) and its f24 literal rules
(src/hvm.rs:1160-1207)."""
from __future__ import annotations

import struct

import numpy as np
import pytest

from conftest import parse_output  # noqa: F401


def defs_of(buf: np.ndarray) -> list[dict]:
    w = [int(x) for x in buf]
    n = w[0]
    at = 1
    out = []
    for _ in range(n):
        fid = w[at]; at += 1
        name = struct.pack("<64I", *w[at:at + 64]).rstrip(b"\0").decode(); at += 64
        safe, rl, nl, vl, root = w[at:at + 5]; at += 5
        rbag = [(w[at + 2 * i], w[at + 2 * i + 1]) for i in range(rl)]; at += 2 * rl
        node = [(w[at + 2 * i], w[at + 2 * i + 1]) for i in range(nl)]; at += 2 * nl
        out.append(dict(fid=fid, name=name, safe=safe, root=root, rbag=rbag, node=node, vars=vl))
    assert at == len(w)
    return out


def port(tag, val):
    return (val << 3) | tag


VAR, REF, ERA, NUM, CON, DUP, OPR, SWI = range(8)


def test_layout_by_hand(hvm):
    # main is fid 0; others follow in sorted-name order (src/ast.rs:532-542).
    code = "@zeta = *\n@main = (a {b $(c a)}) & @alpha ~ (b c)\n@alpha = (x x)\n"
    d = defs_of(hvm.book_from_text(code))
    assert [x["name"] for x in d] == ["main", "alpha", "zeta"]
    m = d[0]
    # DFS pre-order, parent slot first: 0=CON(a, DUP) 1=DUP(b, OPR) 2=OPR(c, a)
    assert m["root"] == port(CON, 0)
    assert m["node"][0] == (port(VAR, 0), port(DUP, 1))
    assert m["node"][1] == (port(VAR, 1), port(OPR, 2))
    assert m["node"][2] == (port(VAR, 2), port(VAR, 0))
    # the redex's tree is numbered after the root's: 3=CON(b, c)
    assert m["rbag"] == [(port(REF, 1), port(CON, 3))]
    assert m["node"][3] == (port(VAR, 1), port(VAR, 2))
    assert m["vars"] == 3
    assert m["safe"] == 0  # DUP inside
    assert d[1]["safe"] == 1 and d[2]["safe"] == 1


def test_par_flag_and_safety_propagation(hvm):
    code = "@main = a &! @f ~ (1 a)\n@f = (x y) & @g ~ (x y)\n@g = ({a b} (a b))\n@h = *\n"
    d = {x["name"]: x for x in defs_of(hvm.book_from_text(code))}
    fst, snd = d["main"]["rbag"][0]
    assert fst == port(REF, d["f"]["fid"] | 0x10000000)  # bit 28 set (src/hvm.rs:203-211)
    assert d["g"]["safe"] == 0
    assert d["f"]["safe"] == 0  # depends on @g
    assert d["main"]["safe"] == 0  # depends on @f
    assert d["h"]["safe"] == 1


def numb_of(hvm, lit: str) -> int:
    d = defs_of(hvm.book_from_text(f"@main = {lit}\n"))
    root = d[0]["root"]
    assert root & 7 == NUM
    return root >> 3


def test_number_literals(hvm):
    assert numb_of(hvm, "42") == (42 << 5) | 1
    assert numb_of(hvm, "0x10") == (16 << 5) | 1
    assert numb_of(hvm, "+7") == (7 << 5) | 2
    assert numb_of(hvm, "-1") == ((0xFFFFFF << 5) | 2)  # a port keeps the low 29 bits
    assert numb_of(hvm, "[+]") == (4 << 5)
    assert numb_of(hvm, "[<<]") == (0x13 << 5)
    assert numb_of(hvm, "[>]") == (0x0F << 5)
    assert numb_of(hvm, "[*2]") == (2 << 5) | 7  # partial: payload 2, op MUL
    assert numb_of(hvm, "[u24]") == (1 << 5)


def f24_bits(hvm, x: float) -> float:
    lit = repr(np.float32(x).item()) if np.isfinite(x) else ("+NaN" if np.isnan(x) else ("+inf" if x > 0 else "-inf"))
    w = numb_of(hvm, lit if "." in lit or "inf" in lit or "NaN" in lit else lit + ".0")
    return np.frombuffer(struct.pack("<I", (w << 3) & 0xFFFFFF00), dtype=np.float32)[0]


def test_f24_roundtrip_known_answers(hvm):
    # Values representable in f24 round-trip exactly (src/hvm.rs:1160-1187).
    for x in [0.0, 1.0, -1.0, 1.1000061, -1.1000061, 2.5, -1.5, 0.25]:
        assert f24_bits(hvm, x) == np.float32(x)
    assert np.isnan(f24_bits(hvm, float("nan")))
    assert f24_bits(hvm, float("inf")) == np.inf
    assert f24_bits(hvm, float("-inf")) == -np.inf


def test_missing_main_and_unbound(hvm):
    with pytest.raises(hvm.HvmError, match="missing `@main` definition"):
        hvm.book_from_text("")
    with pytest.raises(hvm.HvmError, match="Unbound definition: nope"):
        hvm.book_from_text("@main = @nope\n")
    with pytest.raises(hvm.HvmError, match="parse error"):
        hvm.book_from_text("@main = (a\n")


def test_comments_and_whitespace(hvm):
    a = hvm.book_from_text("@main = a // comment\n  & @f ~ (1 a) // more\n@f = (x x)\n")
    b = hvm.book_from_text("@main=a&@f~(1 a)@f=(x x)")
    assert np.array_equal(a, b)


def test_every_reference_program_parses(hvm, ref_programs):
    for p in ref_programs:
        if "build_error" in p:
            with pytest.raises(hvm.HvmError, match=p["build_error"]):
                hvm.book_from_text(p["code"])
        else:
            assert hvm.book_from_text(p["code"]).size > 0


def test_canonical_tree(hvm):
    # vars renamed by first occurrence; f24 in either print format compare equal
    assert hvm.canonical("((a b) (b a))") == hvm.canonical("((x9 y) (y x9))")
    assert hvm.canonical("{2.1500244e+00 *}") == hvm.canonical("{2.1500244 *}")
    assert hvm.canonical("(1 2)") != hvm.canonical("(2 1)")


def test_snapshots_match_reference_c_runtime(hvm, ref_programs):
    # The reference's C runtime, fed this front-end's buffers, reproduces the
    # reference's own snapshots: this pins the front-end.
    checked = 0
    for p in ref_programs:
        if "result" not in p or not p.get("snapshot") or "safety-check" in p["name"]:
            continue
        assert hvm.canonical(p["result"]) == hvm.canonical(p["snapshot"]), p["name"]
        checked += 1
    assert checked >= 10


def test_python_restatement_matches_library(hvm, ref_programs, workloads):
    """oracle/book.py (the front-end restated in Python, used by the bench's
    reference arm so that it never loads this library) and the library's C++
    front-end serialise every reference program, IO program and seeded
    workload to the same words."""
    import json
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    import book as pybook

    io = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "io_programs.json")))
    cases = [p["code"] for p in ref_programs if p["code"].strip()]
    cases += [p["code"] for p in io["programs"]]
    cases += [workloads.tree_sum(12), workloads.bitonic_sort(10), workloads.skewed_fold(10),
              workloads.countdown(1000), workloads.bitonic_sum(6, 7)]
    for code in cases:
        a = hvm.book_from_text(code)
        b = pybook.book_from_text(code)
        assert a.shape == b.shape and (a == b).all()
    with pytest.raises(pybook.ParseError):
        pybook.book_from_text("")


def test_workloads_never_divide(workloads):
    """u24/i24 division and remainder by zero are undefined in the reference
    (SIGFPE on x86) and yield 0 here. The benchmark workloads contain no
    division or remainder operator at all, so they never reach that case."""
    import re
    texts = [workloads.tree_sum(8), workloads.bitonic_sort(6), workloads.skewed_fold(6),
             workloads.countdown(10), workloads.bitonic_sum(6, 7)]
    texts += [code for code, _ in workloads.mixed_batch(64)]
    for code in texts:
        assert not re.search(r"\[:?[/%]", code)


def test_serving_pool_sizes(workloads):
    # The serving workload's templates: the three families in turn, sizes
    # log-uniform in 2^8..2^22 nodes, reproducible from the seed; tree sums of
    # at most 2^21 leaves, bitonic sums of at most 2^14 keys, countdowns of
    # at most 1e5 steps.
    pool = workloads.serving_pool(96)
    assert pool == workloads.serving_pool(96)
    fams = [info["family"] for _, info in pool]
    assert fams == ["tree_sum", "bitonic", "countdown"] * 32
    assert all(8 <= info["log2_size"] <= 22 for _, info in pool)
    assert max(info["depth"] for _, info in pool if info["family"] == "tree_sum") <= 21
    assert max(info["log2n"] for _, info in pool if info["family"] == "bitonic") <= 14
    assert all(10 <= info["length"] <= 100_000 for _, info in pool if info["family"] == "countdown")
