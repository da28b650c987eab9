"""The allocation-free entry point, hvm_gb300_run_noalloc.

Some callers cannot allocate device memory while they evaluate a net: a
host whose device memory is handed out by its own pool or allocator, or an
embedding that must not fail on an allocation. The entry point evaluates a
small net inside a fixed device array the library holds, and must give
exactly what the reference's C runtime gives (its golden normal form and
interaction count) and what the normal entry point gives, on two calls in a
row (the second call runs on an array the first one left dirty).

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SYMS = {1: "[u24]", 2: "[i24]", 3: "[f24]", 4: "[+]", 5: "[-]", 6: "[:-]", 7: "[*]", 8: "[/]", 9: "[:/]",
        10: "[%]", 11: "[:%]", 12: "[=]", 13: "[!]", 14: "[<]", 15: "[>]", 16: "[&]", 17: "[|]", 18: "[^]",
        19: "[<<]", 20: "[:<<]", 21: "[>>]", 22: "[:>>]"}
OPS = {4: "+", 5: "-", 6: ":-", 7: "*", 8: "/", 9: ":/", 10: "%", 11: ":%", 12: "=", 13: "!", 14: "<", 15: ">",
       16: "&", 17: "|", 18: "^", 19: "<<", 20: ":<<", 21: ">>", 22: ":>>"}


def def_names(book: np.ndarray) -> dict[int, str]:
    w = [int(x) for x in book]
    names, at = {}, 1
    for _ in range(w[0]):
        fid = w[at]
        names[fid] = struct.pack("<64I", *w[at + 1:at + 65]).split(b"\0")[0].decode()
        rl, nl = w[at + 66], w[at + 67]
        at += 70 + 2 * (rl + nl)
    return names


def numb_text(w: int) -> str:
    typ = w & 0x1F
    if typ == 0:
        return SYMS.get(w >> 5, "[?]")
    if typ == 1:
        return str(w >> 5)
    if typ == 2:
        v = struct.unpack("<i", struct.pack("<I", (w << 3) & 0xFFFFFFFF))[0] >> 8
        return f"{v:+d}"
    if typ == 3:
        f = struct.unpack("<f", struct.pack("<I", (w << 3) & 0xFFFFFF00))[0]
        if f != f:
            return "+NaN"
        if f in (float("inf"), float("-inf")):
            return "+inf" if f > 0 else "-inf"
        return f"{f:.7e}"
    return f"[{OPS.get(typ, '?')}0x{w >> 5:07X}]"


def render(ports, kids, names) -> str:
    """Prints the breadth-first normal form in the reference's text format."""
    out, stack = [], [0]
    while stack:
        k = stack.pop()
        if isinstance(k, str):
            out.append(k)
            continue
        p = int(ports[k])
        tag, val = p & 7, p >> 3
        if tag >= 4:
            out.append({4: "(", 5: "{", 6: "$(", 7: "?("}[tag])
            c = int(kids[k])
            stack += [{4: ")", 5: "}", 6: ")", 7: ")"}[tag], c + 1, " ", c]
        elif tag == 0:
            out.append(f"x{val:x}")
        elif tag == 1:
            out.append("@" + names[val & 0xFFFFFFF])
        elif tag == 2:
            out.append("*")
        else:
            out.append(numb_text(val))
    return "".join(out)


def run_noalloc(hvm, book: np.ndarray, cap: int = 1 << 16):
    ports = np.zeros(cap, dtype=np.uint32)
    kids = np.zeros(cap, dtype=np.uint32)
    n = ctypes.c_size_t()
    itrs = ctypes.c_uint64()
    err = ctypes.create_string_buffer(512)
    u32p = ctypes.POINTER(ctypes.c_uint32)
    rc = hvm.lib().hvm_gb300_run_noalloc(book.ctypes.data_as(u32p), book.size, ports.ctypes.data_as(u32p),
                                         kids.ctypes.data_as(u32p), cap, ctypes.byref(n), ctypes.byref(itrs),
                                         err, len(err))
    return rc, ports[:n.value], kids[:n.value], itrs.value, err.value.decode()


def programs(ref_programs, workloads, config_goldens):
    """(name, code, golden) with the reference C runtime's result and count:
    `golden` holds `result` (text) or `canonical_sha256`, and `itrs`."""
    # The fixed array is meant for small nets; the large examples (millions
    # of interactions) run through the normal entry point only.
    large = ("sum_tree", "sort_radix", "stress", "sum_rec", "sort_bitonic")
    progs = [(p["name"], p["code"], p) for p in ref_programs
             if "result" in p and not any(x in p["name"] for x in large)]
    progs += [("tree_sum_d12", workloads.tree_sum(12), config_goldens["tree_sum_d12"]),
              ("bitonic_sort_2p8", workloads.bitonic_sort(8), config_goldens["bitonic_sort_2p8"]),
              ("countdown_100000", workloads.countdown(100000), config_goldens["countdown_100000"])]
    return progs


def matches_golden(hvm, canon: str, golden: dict) -> bool:
    if "result" in golden:
        return canon == hvm.canonical(golden["result"])
    return hashlib.sha256(canon.encode()).hexdigest() == golden["canonical_sha256"]


def test_noalloc_matches_goldens_and_normal_entry_point_twice(hvm, ref_programs, workloads, config_goldens):
    progs = programs(ref_programs, workloads, config_goldens)
    # The existing entry point on the same books.
    expected = {}
    with hvm.Runtime(device=0) as rt:
        for name, code, _ in progs:
            rt.load(code)
            st = rt.run()
            expected[name] = (hvm.canonical(rt.result()), st.itrs)
    for name, code, golden in progs:
        book = hvm.book_from_text(code)
        names = def_names(book)
        for call in range(2):
            rc, ports, kids, itrs, err = run_noalloc(hvm, book)
            assert rc == 0, (name, call, err)
            canon = hvm.canonical(render(ports, kids, names))
            assert itrs == golden["itrs"], (name, call)
            assert matches_golden(hvm, canon, golden), (name, call)
            assert (canon, itrs) == expected[name], (name, call)


def test_noalloc_refuses_io_calls(hvm):
    # A program whose normal form asks for an IO call (it opens a file):
    # this entry point has no IO layer, so it answers an error.
    io = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "io_programs.json")))
    code = next(p["code"] for p in io["programs"] if p["name"].endswith("open3.hvm"))
    for _ in range(2):
        rc, _, _, _, err = run_noalloc(hvm, hvm.book_from_text(code))
        assert rc != 0
        assert "IO calls are not supported" in err


def test_noalloc_rejects_books_beyond_its_limits(hvm):
    # 40 nested CON nodes in one definition: more than the fixed array's 32.
    deep = "*"
    for _ in range(40):
        deep = f"({deep} *)"
    book = hvm.book_from_text(f"@main = {deep}\n")
    rc, _, _, _, err = run_noalloc(hvm, book)
    assert rc != 0
    assert "more nodes than the fixed arena allows" in err
