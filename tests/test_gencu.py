"""`hvm gen-cu`: the standalone CUDA program emitter (the reference's
src/main.rs:128-155 splices its runtime and the serialized book into one
`.cu` file). The emitted program must compile on its own with nvcc for
sm_103a and, on a GPU, print what `hvm run-cu` prints for the same file."""
from __future__ import annotations

import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import parse_output

NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17"]


def gen_cu(hvm, path, compiled: bool = False) -> str:
    cmd = [hvm.CLI_PATH, "gen-cu"] + (["--compiled"] if compiled else []) + [str(path)]
    return subprocess.run(cmd, capture_output=True, text=True, check=True).stdout


def compile_cu(src: str, tmp_path, name: str) -> str:
    cu = tmp_path / f"{name}.cu"
    cu.write_text(src)
    exe = str(tmp_path / name)
    r = subprocess.run([NVCC, *NVCC_FLAGS, str(cu), "-o", exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


def test_gen_cu_embeds_the_book_and_compiles(hvm, tmp_path, ref_programs):
    prog = next(p for p in ref_programs if p["name"] == "tests/programs/list.hvm")
    src_file = tmp_path / "list.hvm"
    src_file.write_text(prog["code"])
    out = gen_cu(hvm, src_file)
    # The book buffer is the same words the C ABI receives.
    m = re.search(r"static const uint32_t BOOK_BUF\[(\d+)\] = \{([^}]*)\};", out)
    assert m, "no BOOK_BUF in the emitted program"
    words = [int(x) for x in m.group(2).replace("\n", " ").replace(",", " ").split()]
    assert words == [int(w) for w in hvm.book_from_text(prog["code"])]
    assert int(m.group(1)) == len(words)
    assert "hvm_cu(BOOK_BUF)" in out
    assert '#include "' not in out  # one translation unit, no local headers needed
    compile_cu(out, tmp_path, "list")


def test_compiled_calls_source(hvm, workloads):
    # One straight-line case per def with nodes / links, the def words as
    # immediates relative to the fresh bases, and the book's hash.
    code = workloads.bitonic_sort(8)
    src = hvm.compile_calls(code)
    assert src == hvm.compile_calls(hvm.book_from_text(code))  # text or serialized words
    ndefs = int(hvm.book_from_text(code)[0])
    cases = re.findall(r"^    case (\d+)u:", src, re.M)
    assert 0 < len(cases) <= 2 * ndefs and all(int(c) < ndefs for c in cases)
    assert "compiled_call_nodes" in src and "compiled_call_link" in src
    assert re.search(r"nstore\(d, nb \+ 0u, new_pair\(", src)
    assert re.search(r"uint64_t compiled_book_hash\(\) \{ return 0x[0-9a-f]{16}ull; \}", src)
    with pytest.raises(hvm.HvmError):
        hvm.compile_calls(np.zeros(1, dtype=np.uint32))  # an empty book


def _hot_defs(code: str) -> set[str]:
    # Defs on a cycle of the REF graph, and every def those reach.
    body: dict[str, str] = {}
    name = None
    for line in code.splitlines():
        m = re.match(r"^@([\w.\-/]+)\s*=(.*)$", line)
        if m:
            name = m.group(1)
            body[name] = m.group(2)
        elif name is not None:
            body[name] += " " + line
    refs = {n: set(re.findall(r"@([\w.\-/]+)", b)) & body.keys() for n, b in body.items()}

    def reach(src: str) -> set[str]:
        seen, todo = set(), [src]
        while todo:
            for w in refs[todo.pop()]:
                if w not in seen:
                    seen.add(w)
                    todo.append(w)
        return seen

    cyclic = {n for n in body if n in reach(n)}
    hot = set(cyclic)
    for n in cyclic:
        hot |= reach(n)
    return hot


@pytest.mark.parametrize("make", [lambda W: W.bitonic_sort(8), lambda W: W.tree_sum(12),
                                  lambda W: W.skewed_fold(10), lambda W: W.countdown(1000)],
                         ids=["bitonic_2p8", "tree_sum_d12", "skewed_fold_2p10", "countdown_1000"])
def test_compiled_calls_pick_the_recursive_defs(hvm, workloads, make):
    code = make(workloads)
    src = hvm.compile_calls(code)
    got = set(re.findall(r"^    case \d+u:  // (\S+)$", src, re.M))
    assert got == _hot_defs(code)
    assert "main" not in got


def test_compiled_calls_long_names(hvm, workloads):
    # Def names of any length end up whole in the generated comments, one
    # case per line, so no generated statement can fall into a comment.
    long = "loop_" + "x" * 200
    code = workloads.countdown(1000).replace("@loop", "@" + long)
    src = hvm.compile_calls(code)
    cases = re.findall(r"^    case \d+u:  // (.*)$", src, re.M)
    assert sorted(set(cases)) == sorted({long, long + "__C0"})
    # Apart from the comments, the code is the short-named program's.
    short = hvm.compile_calls(workloads.countdown(1000))
    strip = lambda t: re.sub(r"//[^\n]*", "", t)
    assert strip(src) == strip(short)
    assert "nstore(" in strip(src)


def test_gen_cu_compiled_compiles(hvm, tmp_path, workloads):
    src_file = tmp_path / "bitonic.hvm"
    src_file.write_text(workloads.bitonic_sort(8))
    out = gen_cu(hvm, src_file, compiled=True)
    assert out.index("#define HVM_COMPILED_CALLS") < out.index("namespace hvm")
    assert out.index("compiled_book_hash() {") < out.index("static const uint32_t BOOK_BUF")
    compile_cu(out, tmp_path, "bitonic_compiled")


@pytest.mark.gpu
@pytest.mark.parametrize("compiled", [False, True])
@pytest.mark.parametrize("name", ["tests/programs/list.hvm", "tests/programs/numerics/f24.hvm",
                                  "examples/tuples/tuples.hvm", "examples/sort_bitonic/main.hvm"])
def test_gen_cu_program_matches_run_cu(hvm, tmp_path, ref_programs, name, compiled):
    prog = next(p for p in ref_programs if p["name"] == name)
    src_file = tmp_path / "prog.hvm"
    src_file.write_text(prog["code"])
    exe = compile_cu(gen_cu(hvm, src_file, compiled), tmp_path, "prog")
    got = parse_output(subprocess.run([exe], capture_output=True, text=True, check=True, timeout=300).stdout)
    assert got["itrs"] == prog["itrs"]
    assert hvm.canonical(got["result"]) == hvm.canonical(prog["result"])
