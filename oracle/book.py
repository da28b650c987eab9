"""Pure-Python restatement of the reference's front-end -- test infrastructure.

Turns `.hvm` text into the book buffer that `hvm_c` / `hvm_cu` take, as the
reference's Rust front-end does before either call: parse
(src/ast.rs:44-230), build (src/ast.rs:432-559, safety propagation
src/ast.rs:571-634) and serialize (src/hvm.rs:957-1003). The lexical
primitives come from the reference's parser library TSPL 0.0.13
(Cargo.lock), which is not vendored: `skip_trivia` skips whitespace and `//`
line comments, names are `[A-Za-z0-9_./-]+`, and `parse_u64` reads decimal,
`0x` hex or `0b` binary digits with `_` separators -- the subset every
program of the reference's tests and examples uses.

It exists so that the bench's reference arm and the oracle can serialise
books without loading this repository's library, and so that the tests can
check the library's C++ front-end against a second, independent statement
of the same rules. Nothing in the product imports it.
"""
from __future__ import annotations

import math
import struct

import numpy as np

# Tags (src/hvm.rs:17-26) and numeric type / operator codes (src/hvm.rs:44-68).
VAR, REF, ERA, NUM, CON, DUP, OPR, SWI = range(8)
TY_SYM, TY_U24, TY_I24, TY_F24 = 0, 1, 2, 3
OPS = [  # tried in this order (src/ast.rs:64-84): "<<" before "<", ":-" after "-"
    ("+", 0x04), ("-", 0x05), (":-", 0x06), ("*", 0x07), ("/", 0x08), (":/", 0x09), ("%", 0x0A),
    (":%", 0x0B), ("=", 0x0C), ("!", 0x0D), ("<<", 0x13), (":<<", 0x14), (">>", 0x15), (":>>", 0x16),
    ("<", 0x0E), (">", 0x0F), ("&", 0x10), ("|", 0x11), ("^", 0x12),
]
M32 = 0xFFFFFFFF


class ParseError(ValueError):
    pass


def port(tag: int, val: int) -> int:
    return ((val << 3) | tag) & M32


def pair(fst: int, snd: int) -> int:
    return (snd << 32) | fst


def new_sym(v: int) -> int:
    return ((v << 5) | TY_SYM) & M32


def new_u24(v: int) -> int:
    return ((v << 5) | TY_U24) & M32


def new_i24(v: int) -> int:
    return (((v & M32) << 5) | TY_I24) & M32


def new_f24(val: float) -> int:
    """src/hvm.rs:257-266, round half to even with Rust's bitwise `!`."""
    f = np.float32(val)
    bits = int(np.frombuffer(f.tobytes(), dtype=np.uint32)[0])
    shifted, lost = bits >> 8, bits & 0xFF
    nan = 1 if math.isnan(float(f)) else 0
    shifted += (1 - nan) & ((lost - ((lost >> 7) & (~shifted & M32))) >> 7)
    shifted |= nan
    return ((shifted << 5) | TY_F24) & M32


def partial(a: int, b: int) -> int:
    return ((b & ~0x1F) | (a >> 5)) & M32


class _Parser:
    """src/ast.rs:44-230 over TSPL's primitives."""

    def __init__(self, text: str):
        self.s = text
        self.i = 0

    def fail(self, msg: str):
        line = self.s.count("\n", 0, self.i) + 1
        raise ParseError(f"parse error at line {line}: {msg}")

    def skip_trivia(self):
        s, n = self.s, len(self.s)
        while self.i < n:
            c = s[self.i]
            if c in " \t\n\r\f\v":
                self.i += 1
            elif s.startswith("//", self.i):
                j = s.find("\n", self.i)
                self.i = n if j < 0 else j
            else:
                break

    def peek(self) -> str:
        return self.s[self.i] if self.i < len(self.s) else ""

    def try_consume(self, t: str) -> bool:
        if self.s.startswith(t, self.i):
            self.i += len(t)
            return True
        return False

    def consume(self, t: str):
        self.skip_trivia()
        if not self.try_consume(t):
            self.fail(f"expected '{t}'")

    def name(self) -> str:
        self.skip_trivia()
        j = self.i
        while j < len(self.s) and (self.s[j].isascii() and (self.s[j].isalnum() or self.s[j] in "_.-/")):
            j += 1
        if j == self.i:
            self.fail("expected name")
        out, self.i = self.s[self.i:j], j
        return out

    def _u64(self, s: str, k: int) -> int:
        radix = 10
        if s.startswith("0x", k):
            radix, k = 16, k + 2
        elif s.startswith("0b", k):
            radix, k = 2, k + 2
        v, digits = 0, 0
        for c in s[k:]:
            if c == "_":
                continue
            d = int(c, 16) if c in "0123456789abcdefABCDEF" else 99
            if d >= radix:
                break
            v, digits = (v * radix + d) & 0xFFFFFFFFFFFFFFFF, digits + 1
        if not digits:
            self.fail("expected numeric digit")
        return v

    def numb_lit(self) -> int:
        j = self.i
        while j < len(self.s) and (self.s[j].isascii() and (self.s[j].isalnum() or self.s[j] in "+-.")):
            j += 1
        num, self.i = self.s[self.i:j], j
        if "." in num or "inf" in num or "NaN" in num:
            try:
                val = float(num)
            except ValueError:
                self.fail(f"invalid number literal: {num}")
            return new_f24(val)
        if num[:1] in ("+", "-"):
            v = self._u64(num, 1) & M32
            v = v - (1 << 32) if v >= 1 << 31 else v  # `as i32`
            return new_i24(-v if num[0] == "-" else v)
        return new_u24(self._u64(num, 0) & M32)

    def numb(self) -> int:
        self.skip_trivia()
        if self.peek() != "[":
            return self.numb_lit()
        self.consume("[")
        for cast, ty in (("u24", TY_U24), ("i24", TY_I24), ("f24", TY_F24)):
            if self.try_consume(cast):
                self.consume("]")
                return new_sym(ty)
        for t, code in OPS:
            if self.try_consume(t):
                op = new_sym(code)
                break
        else:
            self.fail("expected operator symbol")
        self.skip_trivia()
        if self.peek() != "]":
            op = partial(op, self.numb_lit())
        self.consume("]")
        return op

    def tree(self):
        self.skip_trivia()
        c = self.peek()
        for opener, closer, kind in (("(", ")", CON), ("{", "}", DUP)):
            if c == opener:
                self.i += 1
                a = self.tree()
                self.skip_trivia()
                b = self.tree()
                self.consume(closer)
                return (kind, a, b)
        for sigil, kind in (("$", OPR), ("?", SWI)):
            if c == sigil:
                self.i += 1
                self.consume("(")
                a = self.tree()
                self.skip_trivia()
                b = self.tree()
                self.consume(")")
                return (kind, a, b)
        if c == "@":
            self.i += 1
            return (REF, self.name())
        if c == "*":
            self.i += 1
            return (ERA,)
        if c and c in "0123456789+-[":
            return (NUM, self.numb())
        return (VAR, self.name())

    def net(self):
        root = self.tree()
        rbag = []
        self.skip_trivia()
        while self.peek() == "&":
            self.consume("&")
            par = self.peek() == "!"
            if par:
                self.consume("!")
            a = self.tree()
            self.consume("~")
            b = self.tree()
            rbag.append((par, a, b))
            self.skip_trivia()
        return root, rbag

    def book(self) -> dict:
        defs = {}
        while True:
            self.skip_trivia()
            if self.i >= len(self.s):
                return defs
            self.consume("@")
            nm = self.name()
            self.consume("=")
            defs[nm] = self.net()


def _refs(t, acc: set):
    stack = [t]
    while stack:
        x = stack.pop()
        if x[0] == REF:
            acc.add(x[1])
        elif x[0] >= CON:
            stack += [x[1], x[2]]


class _Def:
    def __init__(self, name: str):
        self.name, self.safe, self.root = name, True, 0
        self.rbag: list[int] = []
        self.node: list[int] = []
        self.vars: dict[str, int] = {}

    def build(self, t, fids: dict) -> int:
        """src/ast.rs:432-488: DFS pre-order nodes, vars by first occurrence."""
        k = t[0]
        if k == VAR:
            if t[1] not in self.vars:
                self.vars[t[1]] = len(self.vars)
            return port(VAR, self.vars[t[1]])
        if k == REF:
            if t[1] not in fids:
                raise ParseError(f"Unbound definition: {t[1]}")
            return port(REF, fids[t[1]])
        if k == ERA:
            return port(ERA, 0)
        if k == NUM:
            return port(NUM, t[1])
        if k == DUP:
            self.safe = False
        at = len(self.node)
        self.node.append(0)
        a = self.build(t[1], fids)
        b = self.build(t[2], fids)
        self.node[at] = pair(a, b)
        return port(k, at)


def book_from_text(code: str) -> np.ndarray:
    """`Book::parse(code).build().to_buffer()` as u32 words (native endian)."""
    defs = _Parser(code).book()
    fids = {"main": 0}
    for nm in sorted(defs):  # BTreeMap order (bytewise)
        if nm != "main":
            fids[nm] = len(fids)
    if "main" not in defs:
        raise ParseError("missing `@main` definition")
    order = sorted(fids, key=fids.get)
    built = {}
    for nm in order:
        d = _Def(nm)
        root, rbag = defs[nm]
        d.root = d.build(root, fids)
        for par, a, b in rbag:  # src/ast.rs:494-506: slot first, then both trees
            at = len(d.rbag)
            d.rbag.append(0)
            pa, pb = d.build(a, fids), d.build(b, fids)
            if par and pa & 7 == REF:
                pa = port(REF, (pa >> 3) | 0x10000000)
            d.rbag[at] = pair(pa, pb)
        built[nm] = d
    # Safety propagation (src/ast.rs:571-634): unsafe spreads to every def
    # that references an unsafe one, transitively.
    dependents: dict[str, set] = {nm: set() for nm in defs}
    for nm, (root, rbag) in defs.items():
        deps: set = set()
        _refs(root, deps)
        for _, a, b in rbag:
            _refs(a, deps)
            _refs(b, deps)
        for dep in deps:
            dependents[dep].add(nm)
    stack = [nx for nm in defs if not built[nm].safe for nx in dependents[nm]]
    while stack:
        cur = stack.pop()
        if not built[cur].safe:
            continue
        built[cur].safe = False
        stack += list(dependents[cur])
    # src/hvm.rs:957-1003
    out = bytearray(struct.pack("=I", len(order)))
    for fid, nm in enumerate(order):
        d = built[nm]
        raw = nm.encode()
        if len(raw) >= 256:
            raise ParseError(f"Name too long: {nm}")
        out += struct.pack("=I", fid) + raw + bytes(256 - len(raw))
        out += struct.pack("=IIIII", int(d.safe), len(d.rbag), len(d.node), len(d.vars), d.root)
        out += np.asarray(d.rbag + d.node, dtype=np.uint64).tobytes()
    return np.frombuffer(bytes(out), dtype=np.uint32).copy()


def canonical(tree_text: str) -> str:
    """A printed normal form (the text after `Result:`) in the comparison form
    of the reference's test harness (src/tests/run.rs:112-147): variables
    renamed x0, x1, ... by first occurrence, numbers as their 29-bit Numb
    word `#%07X`, so f24 values compare bit for bit whatever their format."""
    p = _Parser(tree_text)
    t = p.tree()
    names: dict[str, int] = {}
    out: list[str] = []
    opener = {CON: "(", DUP: "{", OPR: "$(", SWI: "?("}
    stack = [t]
    while stack:
        x = stack.pop()
        if isinstance(x, str):
            out.append(x)
            continue
        k = x[0]
        if k == VAR:
            out.append("x%d" % names.setdefault(x[1], len(names)))
        elif k == REF:
            out.append("@" + x[1])
        elif k == ERA:
            out.append("*")
        elif k == NUM:
            out.append("#%07X" % (x[1] & 0x1FFFFFFF))
        else:
            out.append(opener[k])
            stack += ["}" if k == DUP else ")", x[2], " ", x[1]]
    return "".join(out)
