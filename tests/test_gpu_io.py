"""IO programs (the reference's tests/programs/io and examples/demo_io): the
evaluator's IO loop reads each IO_CALL back from the device net, runs the host
function (OPEN, READ, WRITE, CLOSE, ...) and writes its result into the net.
Printed output, the normal form and the interaction count must equal the
reference C runtime's on the same files and stdin (tests/golden/io_programs.json,
made by make_golden.py --only-io; the reference harness is tests/run.rs:67-96)."""
from __future__ import annotations

import json
import os
import subprocess

import pytest

from conftest import GOLDEN, parse_output

pytestmark = pytest.mark.gpu

with open(os.path.join(GOLDEN, "io_programs.json")) as _f:
    IO = json.load(_f)


@pytest.mark.parametrize("prog", IO["programs"], ids=[p["name"] for p in IO["programs"]])
def test_io_program_matches_reference(hvm, tmp_path, prog):
    for name, text in IO["files"].items():
        (tmp_path / name).write_text(text)
    src = tmp_path / "prog.hvm"
    src.write_text(prog["code"])
    r = subprocess.run([hvm.CLI_PATH, "run-cu", str(src)], capture_output=True, text=True, cwd=tmp_path,
                       input=IO["stdin"], timeout=300)
    assert r.returncode == 0, r.stderr
    got = parse_output(r.stdout)
    printed = r.stdout[:r.stdout.index("Result: ")]
    assert printed == prog["printed"]
    assert got["itrs"] == prog["itrs"]
    assert hvm.canonical(got["result"]) == hvm.canonical(prog["result"])


def _build_dl_lib(out_dir) -> str:
    """The DL_CALL test library (tests/golden/dl_test.c), built for this host."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib = os.path.join(str(out_dir), IO["dl_lib"])
    subprocess.run(["gcc", "-O2", "-shared", "-fPIC", "-I", os.path.join(root, "include"),
                    os.path.join(GOLDEN, "dl_test.c"), "-o", lib], check=True)
    return lib


@pytest.mark.parametrize("prog", IO["dl"], ids=[p["name"] for p in IO["dl"]])
def test_dl_call_matches_reference(hvm, tmp_path, prog):
    """DL_OPEN + DL_CALL of a library function (src/run.cu:795-813): the GPU
    runtime calls the `*_g` functions through the hvm_gb300_io_* net functions,
    the reference C runtime called their `*_c` twins on its own net; the
    printed output, interaction count and normal form must agree (a missing
    symbol gives the same Err in both)."""
    _build_dl_lib(tmp_path)
    src = tmp_path / "prog.hvm"
    src.write_text(prog["code"])
    r = subprocess.run([hvm.CLI_PATH, "run-cu", str(src)], capture_output=True, text=True, cwd=tmp_path,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    got = parse_output(r.stdout)
    assert r.stdout[:r.stdout.index("Result: ")] == prog["printed"]
    assert got["itrs"] == prog["itrs"]
    assert hvm.canonical(got["result"]) == hvm.canonical(prog["result"])
