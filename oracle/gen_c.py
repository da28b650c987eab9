"""The reference's `hvm gen-c` programs, rebuilt here as a test checker.

TEST INFRASTRUCTURE ONLY: nothing in the product imports or runs this file.

`hvm gen-c FILE` (src/main.rs:100-127) prints the reference's C runtime
(src/hvm.c + src/run.c) with the book's defs compiled into C functions by
`cmp::compile_book(Target::C, ...)` (src/cmp.rs:10-351) and the serialized
book embedded. The reference's compiler is Rust, which is not available
here, so this module restates what compile_book emits for the C target and
splices it into the reference's own sources the way gen-c does:

* per def, `interact_call_<name>` (src/cmp.rs:38-119): the copy optimisation
  for a safe def met by a DUP, one-word allocations of every var and node,
  then the def's root linked to the caller's port through the fast-path
  compiler and the def's redexes linked after it;
* the fast paths of `compile_link_fast` (src/cmp.rs:120-290), tried in this
  order on the def-side port of a link: SWITCH (a `(?((a b) c) c)`-shaped
  CON against a CON whose first port resolves to a number: +3 interactions),
  OPER (an OPR against a number, when its first operand is a number: +1),
  COPY (a DUP against a number: +1), ANNI (a CON against a CON node: +1) and
  VOID (a number or eraser against a number or eraser: +1); otherwise the
  subtree is built and linked (`compile_link_slow`, `link_or_store`);
* `interact_call`, a switch on the def id (src/cmp.rs:10-36).

The emitted C keeps the reference's exact statements, including the mixed
decimal / hexadecimal local-variable names of its SWITCH fast path
(src/cmp.rs:158, 176-177), so the program computes what the reference's
would. The splice follows src/main.rs:110-126: `#define IO` first, the
compiled calls at `///COMPILED_INTERACT_CALL///`, `COMPILED` for
`INTERPRETED`, `BOOK_BUF` (the buffer's bytes) at `//COMPILED_BOOK_BUF//`,
`WITH_MAIN`, TPC_L2, then src/run.c without its `#include "hvm.c"`.

    python oracle/gen_c.py FILE.hvm [--tpc-l2 K] [--run]
"""
from __future__ import annotations

import argparse
import importlib
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# The reference sources as staged by `make -C oracle stage` (or $REF_SRC).
REF_SRC = os.environ.get("REF_SRC", os.path.join(HERE, "_ref", "src"))
OUT_DIR = os.path.join(HERE, "_ref", "genc")

VAR, REF, ERA, NUM, CON, DUP, OPR, SWI = range(8)
TAG_NAMES = ("VAR", "REF", "ERA", "NUM", "CON", "DUP", "OPR", "SWI")


def tag(p: int) -> int:
    return p & 7


def val(p: int) -> int:
    return p >> 3


class Def:
    def __init__(self, name: str, safe: bool, vars_len: int, root: int, rbag: list, node: list):
        self.name, self.safe, self.vars_len, self.root, self.rbag, self.node = name, safe, vars_len, root, rbag, node


def parse_buffer(words) -> list[Def]:
    """Defs of a serialized book (the layout src/hvm.c:1408-1453 reads), by fid."""
    w = [int(x) for x in words]
    at = 1
    defs: dict[int, Def] = {}
    for _ in range(w[0]):
        fid = w[at]
        raw = b"".join(x.to_bytes(4, "little") for x in w[at + 1:at + 65])
        name = raw.split(b"\0", 1)[0].decode()
        safe, rbag_len, node_len, vars_len, root = w[at + 65:at + 70]
        at += 70
        rbag = [(w[at + 2 * i], w[at + 2 * i + 1]) for i in range(rbag_len)]
        at += 2 * rbag_len
        node = [(w[at + 2 * i], w[at + 2 * i + 1]) for i in range(node_len)]
        at += 2 * node_len
        defs[fid] = Def(name, bool(safe), vars_len, root, rbag, node)
    return [defs[f] for f in range(len(defs))]


class DefEmitter:
    """C text of one def's `interact_call_<name>`."""

    def __init__(self, d: Def):
        self.d = d
        self.lines: list[str] = []
        self.names = 0

    def fresh(self) -> str:
        self.names += 1
        return f"k{self.names}"

    def put(self, depth: int, text: str) -> None:
        self.lines.append("  " * depth + text)

    def node_expr(self, depth: int, p: int) -> str:
        """Builds the def-side subtree at port p (children first) and returns
        the C expression of its port."""
        if tag(p) >= CON:
            fst, snd = self.d.node[val(p)]
            e1 = self.node_expr(depth, fst)
            e2 = self.node_expr(depth, snd)
            self.put(depth, f"node_create(net, n{val(p):x}, new_pair({e1},{e2}));")
            return f"new_port({TAG_NAMES[tag(p)]},n{val(p):x})"
        if tag(p) == VAR:
            return f"new_port(VAR,v{val(p):x})"
        return f"new_port({TAG_NAMES[tag(p)]},0x{val(p):08x})"

    def link_or_store(self, depth: int, a: str, b: str) -> None:
        self.put(depth, f"if ({b} != NONE) {{")
        self.put(depth + 1, f"link(net, tm, {a}, {b});")
        self.put(depth, "} else {")
        self.put(depth + 1, f"{b} = {a};")
        self.put(depth, "}")

    def link_slow(self, depth: int, a: int, b: str) -> None:
        self.link_or_store(depth, self.node_expr(depth, a), b)

    def _switch_shape(self, a: int):
        # (?((a111 a112) a12) a2) with a12 the same var as a2
        if tag(a) != CON:
            return None
        a1, a2 = self.d.node[val(a)]
        if tag(a1) != SWI:
            return None
        a11, a12 = self.d.node[val(a1)]
        if tag(a11) != CON or tag(a2) != VAR or a12 != a2:
            return None
        return a1, a2, a11, a12

    def link_fast(self, depth: int, a: int, b: str) -> None:
        """Links def-side port a to the C variable b, reducing on the spot
        when b already holds what a's shape needs."""
        shape = self._switch_shape(a)
        if shape:
            a1, a2, a11, a12 = shape
            a111, a112 = self.d.node[val(a11)]
            op, bv, x1, x2, nu = (self.fresh() for _ in range(5))
            self.put(depth, f"bool {op} = 0;")
            self.put(depth, f"Pair {bv} = 0;")
            self.put(depth, f"Port {nu} = NONE;")
            self.put(depth, f"Port {x1} = NONE;")
            self.put(depth, f"Port {x2} = NONE;")
            self.put(depth, f"if (get_tag({b}) == CON) {{")
            self.put(depth + 1, f"{bv} = node_load(net, get_val({b}));")
            self.put(depth + 1, f"{nu} = enter(net,get_fst({bv}));")
            self.put(depth + 1, f"if (get_tag({nu}) == NUM) {{")
            self.put(depth + 2, "tm->itrs += 3;")
            self.put(depth + 2, f"vars_take(net, v{val(a2)});")
            self.put(depth + 2, f"{op} = 1;")
            self.put(depth + 2, f"if (get_u24(get_val({nu})) == 0) {{")
            self.put(depth + 3, f"node_take(net, get_val({b}));")
            self.put(depth + 3, f"{x1} = get_snd({bv});")
            self.put(depth + 3, f"{x2} = new_port(ERA,0);")
            self.put(depth + 2, "} else {")
            self.put(depth + 3, f"node_store(net, get_val({b}), new_pair(new_port(NUM,new_u24(get_u24(get_val({nu}))-1)), "
                                f"get_snd({bv})));")
            self.put(depth + 3, f"{x1} = new_port(ERA,0);")
            self.put(depth + 3, f"{x2} = {b};")
            self.put(depth + 2, "}")
            self.put(depth + 1, "} else {")
            self.put(depth + 2, f"node_store(net, get_val({b}), new_pair({nu},get_snd({bv})));")
            self.put(depth + 1, "}")
            self.put(depth, "}")
            self.link_fast(depth, a111, x1)
            self.link_fast(depth, a112, x2)
            self.put(depth, f"if (!{op}) {{")
            self.put(depth + 1, f"node_create(net, n{val(a):x}, new_pair(new_port(SWI,n{val(a1)}),new_port(VAR,v{val(a2)})));")
            self.put(depth + 1, f"node_create(net, n{val(a1):x}, new_pair(new_port(CON,n{val(a11)}),new_port(VAR,v{val(a12)})));")
            self.put(depth + 1, f"node_create(net, n{val(a11):x}, new_pair({x1},{x2}));")
            self.link_or_store(depth + 1, f"new_port(CON, n{val(a):x})", b)
            self.put(depth, "}")
            return
        if tag(a) == OPR:
            a1, a2 = self.d.node[val(a)]
            op = self.fresh()
            x1 = self.node_expr(depth, a1)
            x2 = self.fresh()
            self.put(depth, f"bool {op} = 0;")
            self.put(depth, f"Port {x2} = NONE;")
            self.put(depth, f"if (get_tag({b}) == NUM && get_tag({x1}) == NUM) {{")
            self.put(depth + 1, "tm->itrs += 1;")
            self.put(depth + 1, f"{op} = 1;")
            self.put(depth + 1, f"{x2} = new_port(NUM, operate(get_val({b}), get_val({x1})));")
            self.put(depth, "}")
            self.link_fast(depth, a2, x2)
            self.put(depth, f"if (!{op}) {{")
            self.put(depth + 1, f"node_create(net, n{val(a):x}, new_pair({x1},{x2}));")
            self.link_or_store(depth + 1, f"new_port(OPR, n{val(a):x})", b)
            self.put(depth, "}")
            return
        if tag(a) in (DUP, CON):
            p1, p2 = self.d.node[val(a)]
            anni = tag(a) == CON
            op = self.fresh()
            bv = self.fresh() if anni else None
            x1, x2 = self.fresh(), self.fresh()
            self.put(depth, f"bool {op} = 0;")
            if anni:
                self.put(depth, f"Pair {bv} = 0;")
            self.put(depth, f"Port {x1} = NONE;")
            self.put(depth, f"Port {x2} = NONE;")
            if anni:
                self.put(depth, f"if (get_tag({b}) == CON && node_load(net, get_val({b})) != 0) {{")
                self.put(depth + 1, "tm->itrs += 1;")
                self.put(depth + 1, f"{op} = 1;")
                self.put(depth + 1, f"{bv} = node_take(net, get_val({b}));")
                self.put(depth + 1, f"{x1} = get_fst({bv});")
                self.put(depth + 1, f"{x2} = get_snd({bv});")
            else:
                self.put(depth, f"if (get_tag({b}) == NUM) {{")
                self.put(depth + 1, "tm->itrs += 1;")
                self.put(depth + 1, f"{op} = 1;")
                self.put(depth + 1, f"{x1} = {b};")
                self.put(depth + 1, f"{x2} = {b};")
            self.put(depth, "}")
            self.link_fast(depth, p2, x2)
            self.link_fast(depth, p1, x1)
            self.put(depth, f"if (!{op}) {{")
            self.put(depth + 1, f"node_create(net, n{val(a):x}, new_pair({x1},{x2}));")
            self.link_or_store(depth + 1, f"new_port({'CON' if anni else 'DUP'},n{val(a):x})", b)
            self.put(depth, "}")
            return
        if tag(a) in (NUM, ERA):
            self.put(depth, f"if (get_tag({b}) == ERA || get_tag({b}) == NUM) {{")
            self.put(depth + 1, "tm->itrs += 1;")
            self.put(depth, "} else {")
            self.link_slow(depth + 1, a, b)
            self.put(depth, "}")
            return
        self.link_slow(depth, a, b)

    def function(self, fun: str) -> str:
        d = self.d
        self.put(0, f"bool interact_call_{fun}(Net *net, TM *tm, Port a, Port b) {{")
        if d.safe:
            self.put(1, "if (get_tag(b) == DUP) {")
            self.put(2, "return interact_eras(net, tm, a, b);")
            self.put(1, "}")
        self.put(1, "u32 vl = 0;")
        self.put(1, "u32 nl = 0;")
        for i in range(d.vars_len):
            self.put(1, f"Val v{i:x} = vars_alloc_1(net, tm, &vl);")
        for i in range(len(d.node)):
            self.put(1, f"Val n{i:x} = node_alloc_1(net, tm, &nl);")
        missing = "".join(f" || !v{i:x}" for i in range(d.vars_len)) + \
            "".join(f" || !n{i:x}" for i in range(len(d.node)))
        self.put(1, f"if (0{missing}) {{")
        self.put(2, "return false;")
        self.put(1, "}")
        for i in range(d.vars_len):
            self.put(1, f"vars_create(net, v{i:x}, NONE);")
        self.link_fast(1, d.root, "b")
        for fst, snd in d.rbag:
            e1 = self.node_expr(1, fst)
            e2 = self.node_expr(1, snd)
            self.put(1, f"link(net, tm, {e1}, {e2});")
        self.put(1, "return true;")
        self.put(0, "}")
        return "\n".join(self.lines) + "\n"


def c_name(name: str) -> str:
    return name.replace("/", "_").replace(".", "_").replace("-", "_")


def compile_book_c(defs: list[Def]) -> str:
    """What cmp::compile_book(Target::C, book) returns for these defs."""
    out = [DefEmitter(d).function(c_name(d.name)) + "\n" for d in defs]
    out.append("bool interact_call(Net *net, TM *tm, Port a, Port b) {\n")
    out.append("  u32 fid = get_val(a) & 0xFFFFFFF;\n  switch (fid) {\n")
    for fid, d in enumerate(defs):
        out.append(f"    case {fid}: return interact_call_{c_name(d.name)}(net, tm, a, b);\n")
    out.append("    default: return false;\n  }\n}")
    return "".join(out)


def gen_c_program(words, tpc_l2: int = 0) -> str:
    """The text `hvm gen-c` prints for a serialized book."""
    hvm_c = open(os.path.join(REF_SRC, "hvm.c")).read()
    run_c = open(os.path.join(REF_SRC, "run.c")).read()
    raw = b"".join(int(x).to_bytes(4, "little") for x in words)
    book_buf = "static const u8 BOOK_BUF[] = {" + ", ".join(str(b) for b in raw) + "};"
    text = "#define IO\n\n" + hvm_c
    text = text.replace("///COMPILED_INTERACT_CALL///", compile_book_c(parse_buffer(words)))
    text = text.replace("#define INTERPRETED", "#define COMPILED")
    text = text.replace("//COMPILED_BOOK_BUF//", book_buf)
    text = text.replace("#define WITHOUT_MAIN", "#define WITH_MAIN")
    text = text.replace("#define TPC_L2 0", f"#define TPC_L2 {tpc_l2}")
    text = text + "\n\n" + run_c
    return text.replace('#include "hvm.c"', "")


def build_and_run(words, name: str, tpc_l2: int = 0, timeout: float = 600) -> dict:
    """Compiles the gen-c program for a book into oracle/_ref/genc/ and runs
    it: its `Result:` text and `- ITRS` count."""
    os.makedirs(OUT_DIR, exist_ok=True)
    src = os.path.join(OUT_DIR, f"{name}_t{tpc_l2}.c")
    exe = src[:-2]
    with open(src, "w") as f:
        f.write(gen_c_program(words, tpc_l2))
    cc = os.environ.get("CC", "gcc")
    r = subprocess.run([cc, "-O2", "-w", "-o", exe, src, "-lm", "-lpthread", "-ldl"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"gen-c program for {name} does not compile:\n{r.stderr[-3000:]}")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=timeout)
    res = re.search(r"^Result: (.*)$", r.stdout, re.M)
    itrs = re.search(r"^- ITRS: (\d+)$", r.stdout, re.M)
    if r.returncode != 0 or not res or not itrs:
        raise RuntimeError(f"gen-c program for {name} failed: rc={r.returncode}\n{r.stdout[-2000:]}{r.stderr[-2000:]}")
    return {"result": res.group(1), "itrs": int(itrs.group(1))}


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("file")
    ap.add_argument("--tpc-l2", type=int, default=0)
    ap.add_argument("--run", action="store_true", help="compile and run instead of printing the program")
    args = ap.parse_args()
    sys.path.insert(0, ROOT)
    hvm = importlib.import_module("lambdavm-rust_gb300")
    words = hvm.book_from_text(open(args.file).read())
    if args.run:
        out = build_and_run(words, os.path.splitext(os.path.basename(args.file))[0], args.tpc_l2)
        print(f"Result: {out['result']}\n- ITRS: {out['itrs']}")
    else:
        sys.stdout.write(gen_c_program(words, args.tpc_l2))


if __name__ == "__main__":
    main()
