"""The C-ABI library loads and exports every symbol include/hvm_gb300.h
declares (no device calls: this runs without a GPU)."""
from __future__ import annotations

import ctypes
import os
import re
import subprocess

from conftest import ROOT


def declared_functions() -> set[str]:
    text = open(os.path.join(ROOT, "include", "hvm_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(hvm_\w+)\s*\(", text))


def test_header_matches_exports(hvm):
    decl = declared_functions()
    assert decl == set(hvm.EXPORTED_SYMBOLS)
    L = ctypes.CDLL(hvm.LIB_PATH)
    for name in decl:
        assert hasattr(L, name), name
    nm = subprocess.run(["nm", "-D", "--defined-only", hvm.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (\w+)$", nm, re.M))
    assert decl <= exported


def test_default_config(hvm):
    cfg = hvm.Config()
    hvm.lib().hvm_gb300_default_config(ctypes.byref(cfg))
    assert cfg.threads_per_block % 32 == 0
    assert cfg.node_log2 <= 29 and cfg.vars_log2 <= 29
    assert cfg.stack_cap > 0


def test_cli_book_matches_library(hvm, tmp_path):
    src = tmp_path / "p.hvm"
    src.write_text("@main = a & @f ~ (1 a)\n@f = (x x)\n")
    out = tmp_path / "p.bin"
    subprocess.run([hvm.CLI_PATH, "book", str(src), str(out)], check=True)
    import numpy as np
    assert np.array_equal(np.fromfile(out, dtype=np.uint32), hvm.book_from_text(src.read_text()))


def test_committed_policy_weights_are_well_formed(hvm):
    import importlib
    train = importlib.import_module("lambdavm-rust_gb300.train_policy")
    w = train.load_weights()
    assert w.shape == (hvm.POLICY_PARAMS,)
    assert hvm.POLICY_PARAMS == 5443


def test_ctypes_mirrors_match_the_header(hvm, tmp_path):
    # The Python structs must have the C header's layout: compare sizes
    # (and the offset of the last field) with a probe compiled against it.
    import ctypes
    import os
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    src = tmp_path / "probe.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "hvm_gb300.h"\n'
                   'int main(void) { printf("%zu %zu %zu %zu %zu\\n", sizeof(hvm_gb300_config),'
                   ' offsetof(hvm_gb300_config, turn_budget_cap), sizeof(hvm_gb300_stats),'
                   ' sizeof(hvm_gb300_turn), offsetof(hvm_gb300_turn, outputs)); return 0; }\n')
    exe = tmp_path / "probe"
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == [ctypes.sizeof(hvm.Config), hvm.Config.turn_budget_cap.offset, ctypes.sizeof(hvm._Stats),
                   ctypes.sizeof(hvm.Turn), hvm.Turn.outputs.offset]


def test_port64_library_exports_and_refuses_32bit_calls(hvm):
    # The 64-bit port build exports the same C ABI; the no-alloc entry point,
    # whose output ports are 32-bit, refuses before touching a device.
    L = hvm.lib64()
    nm = subprocess.run(["nm", "-D", "--defined-only", hvm.LIB64_PATH], capture_output=True, text=True).stdout
    assert declared_functions() <= set(re.findall(r" T (\w+)$", nm, re.M))
    import numpy as np
    book = hvm.book_from_text("@main = 1\n")
    out = np.zeros(16, dtype=np.uint32)
    err = ctypes.create_string_buffer(256)
    n, itrs = ctypes.c_size_t(), ctypes.c_uint64()
    u32p = ctypes.POINTER(ctypes.c_uint32)
    rc = L.hvm_gb300_run_noalloc(book.ctypes.data_as(u32p), book.size, out.ctypes.data_as(u32p),
                                 out.ctypes.data_as(u32p), 8, ctypes.byref(n), ctypes.byref(itrs), err, 256)
    assert rc == -1 and b"64-bit" in err.value
