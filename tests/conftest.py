"""Shared test fixtures.

`-m "not gpu"` tests run anywhere (front-end, C ABI exports, the CPU oracle
against the reference's golden vectors). `-m gpu` tests run the sm_103a
evaluator through the C ABI and compare with the oracle and the goldens.
"""
from __future__ import annotations

import importlib
import json
import os
import re
import subprocess
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
ORACLE_BIN = os.path.join(ROOT, "oracle", "_build", "hvm_oracle")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a evaluator)")
    config.addinivalue_line("markers", "slow: full-size workloads")


def _build_once():
    build = importlib.import_module("lambdavm-rust_gb300.build")
    build.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)


@pytest.fixture(scope="session")
def hvm():
    _build_once()
    return importlib.import_module("lambdavm-rust_gb300")


@pytest.fixture(scope="session")
def workloads():
    return importlib.import_module("lambdavm-rust_gb300.workloads")


@pytest.fixture(scope="session")
def ref_programs():
    with open(os.path.join(GOLDEN, "reference_programs.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def config_goldens():
    with open(os.path.join(GOLDEN, "configs.json")) as f:
        return json.load(f)


def parse_output(text: str) -> dict:
    res = re.search(r"^Result: (.*)$", text, re.M)
    itrs = re.search(r"^- ITRS: (\d+)$", text, re.M)
    return {"result": res.group(1) if res else None, "itrs": int(itrs.group(1)) if itrs else None}


@pytest.fixture(scope="session")
def oracle(hvm):
    """Runs the CPU oracle (oracle/hvm_oracle.c) on `.hvm` text."""

    def run(code: str, threads: int = 1, timeout: float = 600) -> dict:
        buf = hvm.book_from_text(code)
        with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as f:
            buf.tofile(f.name)
            path = f.name
        try:
            r = subprocess.run([ORACLE_BIN, "-t", str(threads), path], capture_output=True, text=True,
                               timeout=timeout)
        finally:
            os.unlink(path)
        assert r.returncode == 0, r.stderr
        return parse_output(r.stdout)

    return run
