"""The 64-bit port encoding against the reference's 32-bit one, on the host
(no GPU): lambdavm-rust_gb300/csrc/hvm_defs.h compiled twice, with and
without HVM_PORT64. A number port must hold the same 29-bit Numb in both --
u24/i24 results wrap at 24 bits where the reference's (numb << 3) leaves its
32-bit word -- and node pairs and var/node ports must round-trip with
values past the 32-bit port's range."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "lambdavm-rust_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include "hvm_defs.h"
using namespace hvm;
int main() {
  // A seeded walk over operand pairs and every u24/i24 operator.
  unsigned long long s = 0x9E3779B97F4A7C15ull;
  auto next = [&]() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return (uint32_t)s; };
  const uint32_t ops[] = {OP_ADD, OP_SUB, FP_SUB, OP_MUL, OP_DIV, FP_DIV, OP_REM, FP_REM, OP_EQ, OP_NEQ,
                          OP_LT, OP_GT, OP_AND, OP_OR, OP_XOR, OP_SHL, FP_SHL, OP_SHR, FP_SHR};
  unsigned long long h = 1469598103934665603ull;
  for (int i = 0; i < 200000; i++) {
    const uint32_t op = ops[next() % 19];
    const bool sgn = next() & 1;
    const uint32_t x = next() & 0xFFFFFF, y = (next() & 0xFFFFFF) | 1;  // y != 0: no division by zero
    const Numb a = sgn ? new_i24((int32_t)(x << 8) >> 8) : new_u24(x);
    const Numb b = sgn ? new_i24((int32_t)(y << 8) >> 8) : new_u24(y);
    const Numb sym = (op << 5) | TY_SYM;
    const Numb partial = operate(sym, a);
    const Numb r = operate(partial, b);
    const Port p = new_port(NUM, r);
    const uint32_t v = (uint32_t)get_val(p);  // the Numb a number port carries
    h = (h ^ v) * 1099511628211ull;
  }
  printf("numbers %016llx\n", h);
  // Pairs and pointer ports round-trip at the largest indices of this width.
  const Val big = PORT_BITS == 64 ? 0xFFFFFFF0ull : 0x1FFFFFF0u;
  const Port a = new_port(CON, big), b = new_port(VAR, big + 7);
  const Pair q = new_pair(a, b);
  const bool ok = get_fst(q) == a && get_snd(q) == b && get_val(a) == big && get_tag(b) == VAR &&
                  get_val(ROOT) == ROOT_VAR && get_tag(ROOT) == VAR && NONE != ROOT;
  printf("pairs %s\n", ok ? "ok" : "bad");
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="no host C++ compiler")
def test_port64_numbers_and_pairs_match_32bit(tmp_path):
    src = tmp_path / "enc.cpp"
    src.write_text(PROGRAM)
    outs = {}
    for name, defs in (("p32", []), ("p64", ["-DHVM_PORT64"])):
        exe = tmp_path / name
        subprocess.run(["g++", "-O2", "-std=c++17", *defs, "-I", CSRC, str(src), "-o", str(exe)], check=True)
        outs[name] = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()
    assert outs["p32"][0] == outs["p64"][0]  # the same 29-bit Numbs in number ports
    assert outs["p32"][1] == outs["p64"][1] == "pairs ok"
