"""Builds the native parts of the package in-tree.

  libhvm_gb300.so   the C-ABI library (front-end + sm_103a evaluator + runtime)
  hvm               the command-line driver (`hvm run-cu FILE`, `hvm gen-cu FILE`)

Compiled for sm_103a only (`-gencode arch=compute_103a,code=sm_103a`), with
translation units built in parallel. Runs the same on x86_64 (cross-compile,
no GPU needed) and on the aarch64 GPU host.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libhvm_gb300.so")
# The same runtime over 64-bit ports (HVM_PORT64: 128-bit node pairs, spaces
# of up to 2^32 words); the front-end and the MLP kernels are shared objects.
LIB64 = os.path.join(PKG, "libhvm_gb300_p64.so")
CLI = os.path.join(PKG, "hvm")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O3", "-std=c++17", "-I" + INCLUDE, "-I" + CSRC]

LIB_SOURCES = ["frontend.cpp", "runtime.cu", "mlp.cu", "peaks.cu"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]


def _compile(src: str, port64: bool = False) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + (".p64.o" if port64 else ".o"))
    defs = ["-DHVM_PORT64"] if port64 else []
    if _stale(obj, [path] + _headers()):
        if src.endswith(".cu"):
            _run([NVCC, *ARCH, "-lineinfo", *CXXFLAGS, *defs, "-Xcompiler", "-fPIC", "-c", path, "-o", obj])
        else:
            _run([NVCC, *CXXFLAGS, *defs, "-Xcompiler", "-fPIC", "-c", path, "-o", obj])
    return obj


STANDALONE_ROOT = "runtime.cu"
STANDALONE_INC = os.path.join(BUILD, "standalone_source.inc")
RAW_DELIM = "HVMGB300SRC"


def standalone_source() -> str:
    """The evaluator runtime as one CUDA translation unit: runtime.cu with
    every local `#include "..."` replaced by the file's text (each file once),
    for `hvm gen-cu` to print around an embedded book."""
    seen: set[str] = set()

    def expand(name: str) -> str:
        for d in (CSRC, INCLUDE):
            path = os.path.join(d, name)
            if os.path.exists(path):
                break
        else:
            raise FileNotFoundError(name)
        if path in seen:
            return ""
        seen.add(path)
        out = []
        for line in open(path).read().splitlines():
            st = line.strip()
            if st == "#pragma once":
                continue
            if st.startswith('#include "') and st.endswith('"'):
                out.append(expand(st[len('#include "'):-1]))
                continue
            out.append(line)
        return "\n".join(out)

    src = expand(STANDALONE_ROOT)
    if ")" + RAW_DELIM + '"' in src:
        raise RuntimeError("raw-string delimiter occurs in the sources")
    return src


def _write_standalone() -> None:
    text = 'static const char HVM_STANDALONE_SOURCE[] = R"' + RAW_DELIM + "(" + standalone_source() + ")" + \
        RAW_DELIM + '";\n'
    if not os.path.exists(STANDALONE_INC) or open(STANDALONE_INC).read() != text:
        with open(STANDALONE_INC, "w") as f:
            f.write(text)


def build(verbose: bool = False) -> str:
    """Compiles the library and the CLI if any source changed; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    _write_standalone()
    with ThreadPoolExecutor(max_workers=max(2, len(LIB_SOURCES) + 1)) as ex:
        jobs = [ex.submit(_compile, src) for src in LIB_SOURCES]
        job64 = ex.submit(_compile, "runtime.cu", True)
        objs = [j.result() for j in jobs]
        obj64 = job64.result()
    if _stale(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    objs64 = [obj64 if o.endswith("runtime.cu.o") else o for o in objs]
    if _stale(LIB64, objs64):
        _run([NVCC, *ARCH, "-shared", "-o", LIB64, *objs64, "-lcudart"])
    cli_src = os.path.join(CSRC, "hvm_cli.cpp")
    if os.path.exists(cli_src) and _stale(CLI, [cli_src, LIB, STANDALONE_INC] + _headers()):
        _run([NVCC, *CXXFLAGS, "-I" + BUILD, "-o", CLI, cli_src, "-L" + PKG, "-lhvm_gb300",
              "-Xlinker", "-rpath=$ORIGIN"])
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
