"""Seeded synthetic HVM2 programs for the benchmark configurations.

The reference publishes no benchmark suite (its `hvm-bench` repository is not
part of it); these generators produce `.hvm` IR in the style of the
reference's own examples (examples/sum_tree, examples/sort_bitonic,
examples/stress), with input data embedded as a perfect binary tree of CON
nodes split into REF'd sub-definitions of at most 31 CON nodes each (the
reference CUDA loader rejects definitions with more than 64 nodes,
src/hvm.cu:1922-1930).

Workloads:
  tree_sum(20)       sum(d) = d==0 ? 1 : sum(d-1)+sum(d-1)       -> 1048576
  bitonic_sort(16)   sort of 2^16 PCG32 u24 keys, returns the sorted tree
  skewed_fold(18)    2^18 countdown loops of Geometric(1/64) length capped
                     at 2^16, results summed in a balanced tree    -> 2^18
  mixed_batch(...)   per-net seeds for the 4096-net mixed batch
"""
from __future__ import annotations

import math

# PCG32 (O'Neill, "PCG: A Family of Simple Fast Space-Efficient Statistically
# Good Algorithms for Random Number Generation", 2014): 64-bit LCG state,
# XSH-RR output.
PCG_MULT = 6364136223846793005
PCG_DEFAULT_STATE = 0x853C49E6748FEA9B
PCG_DEFAULT_SEQ = 0xDA3E39CB94B95BDB
M64 = (1 << 64) - 1


class PCG32:
    def __init__(self, initstate: int = PCG_DEFAULT_STATE, initseq: int = PCG_DEFAULT_SEQ):
        self.state = 0
        self.inc = ((initseq << 1) | 1) & M64
        self.next()
        self.state = (self.state + initstate) & M64
        self.next()

    def next(self) -> int:
        old = self.state
        self.state = (old * PCG_MULT + self.inc) & M64
        xorshifted = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xorshifted >> rot) | (xorshifted << ((-rot) & 31))) & 0xFFFFFFFF

    def uniform(self) -> float:
        """Uniform in [0, 1) from 32 random bits."""
        return self.next() / 4294967296.0


def _data_tree(prefix: str, leaves: list[str], chunk: int = 5) -> tuple[str, list[str]]:
    """Embeds `leaves` (a power of two) as a perfect CON tree split into defs.

    Returns (root tree text, list of `@name = tree` lines). Each def holds at
    most `chunk` levels (2^chunk - 1 CON nodes); deeper subtrees are REFs.
    """
    n = len(leaves)
    depth = int(math.log2(n))
    assert 1 << depth == n, "leaf count must be a power of two"
    defs: list[str] = []

    def inline(parts: list[str]) -> str:
        while len(parts) > 1:
            parts = [f"({parts[i]} {parts[i + 1]})" for i in range(0, len(parts), 2)]
        return parts[0]

    def build(lo: int, d: int) -> str:
        top = d % chunk or min(chunk, d)
        rest = d - top
        parts = []
        for j in range(1 << top):
            start = lo + (j << rest)
            if rest == 0:
                parts.append(leaves[start])
            else:
                name = f"{prefix}.{rest}.{start}"
                defs.append(f"@{name} = {build(start, rest)}")
                parts.append("@" + name)
        return inline(parts)

    if depth == 0:
        return leaves[0], defs
    return build(0, depth), defs


def tree_sum(depth: int = 20) -> str:
    """sum(d) = d==0 ? 1 : sum(d-1) + sum(d-1), in the split-def style of
    examples/stress/main.hvm:1-8. Normal form: 2^depth."""
    return "\n".join([
        f"@main = a & @sum ~ ({depth} a)",
        "@sum = (?((1 @sum__C0) a) a)",
        "@sum__C0 = ({a b} d)",
        "  &! @sum ~ (a $([+] $(c d)))",
        "  &! @sum ~ (b c)",
        "",
    ])


BITONIC_DEFS = """\
@down = (?(((a (* a)) @down__C0) (b (c d))) (c (b d)))
@down__C0 = ({a e} ((c g) ({b f} (d h))))
  &! @flow ~ (a (b (c d)))
  &! @flow ~ (e (f (g h)))
@flow = (?(((a (* a)) @flow__C0) (b (c d))) (c (b d)))
@flow__C0 = ({$([+1] a) c} ((e f) ({b d} h)))
  & @down ~ (a (b (g h)))
  & @warp ~ (c (d (e (f g))))
@sort = (?(((a (* a)) @sort__C0) (b (c d))) (c (b d)))
@sort__C0 = ({$([+1] a) {c f}} ((d g) (b i)))
  & @flow ~ (a (b ((e h) i)))
  &! @sort ~ (c (0 (d e)))
  &! @sort ~ (f (1 (g h)))
@swap = (?((@swap__C0 @swap__C1) (a (b c))) (b (a c)))
@swap__C0 = (b (a (a b)))
@swap__C1 = (* (a (b (a b))))
@warp = (?((@warp__C0 @warp__C1) (a (b (c d)))) (c (b (a d))))
@warp__C0 = ({a e} ({$([>] $(a b)) d} ($([^] $(b c)) f)))
  & @swap ~ (c (d (e f)))
@warp__C1 = ({a f} ((d i) ((c h) ({b g} ((e j) (k l))))))
  &! @warp ~ (f (g (h (i (j l)))))
  &! @warp ~ (a (b (c (d (e k)))))
"""


def pcg_keys(n: int, seed: int = PCG_DEFAULT_STATE, seq: int = PCG_DEFAULT_SEQ) -> list[int]:
    rng = PCG32(seed, seq)
    return [rng.next() & 0xFFFFFF for _ in range(n)]


def bitonic_sort(log2n: int = 16, seed: int = PCG_DEFAULT_STATE, seq: int = PCG_DEFAULT_SEQ) -> str:
    """Bitonic sort (the sort/flow/down/warp/swap functions of
    examples/sort_bitonic/main.hvm) of 2^log2n PCG32 u24 keys embedded as a
    depth-log2n CON tree; the normal form is the sorted tree."""
    keys = pcg_keys(1 << log2n, seed, seq)
    root, defs = _data_tree("K", [str(k) for k in keys])
    lines = [f"@main = a & @sort ~ ({log2n} (0 ({root} a)))", BITONIC_DEFS] + defs
    return "\n".join(lines) + "\n"


def geometric_lengths(n: int, p: float = 1.0 / 64, cap: int = 1 << 16,
                      seed: int = PCG_DEFAULT_STATE, seq: int = PCG_DEFAULT_SEQ) -> list[int]:
    """Lengths ~ Geometric(p) on {1, 2, ...} (mean 1/p), capped, by inversion."""
    rng = PCG32(seed, seq)
    out = []
    lq = math.log1p(-p)
    for _ in range(n):
        u = rng.uniform()
        k = int(math.floor(math.log1p(-u) / lq)) + 1
        out.append(min(k, cap))
    return out


def skewed_fold(log2n: int = 18, seed: int = PCG_DEFAULT_STATE, seq: int = PCG_DEFAULT_SEQ,
                p: float = 1.0 / 64, cap: int = 1 << 16) -> str:
    """A fold over 2^log2n elements; element i runs a countdown loop
    (examples/stress/main.hvm:10-13) of a seeded geometric length and yields
    1; the fold sums them in a balanced tree. Normal form: 2^log2n."""
    lens = geometric_lengths(1 << log2n, p, cap, seed, seq)
    root, defs = _data_tree("L", [str(x) for x in lens])
    lines = [
        f"@main = a & @fold ~ ({log2n} ({root} a))",
        "@fold = (?((@leaf @fold__C0) a) a)",
        "@fold__C0 = ({a c} ((b d) f))",
        "  &! @fold ~ (a (b $([+] $(e f))))",
        "  &! @fold ~ (c (d e))",
        "@leaf = (n r) & @loop ~ (n $([+1] r))",
        "@loop = (?((0 @loop__C0) a) a)",
        "@loop__C0 = a & @loop ~ a",
    ] + defs
    return "\n".join(lines) + "\n"


def countdown(length: int) -> str:
    """One countdown loop of `length` steps (examples/stress/main.hvm:10-13)."""
    return "\n".join([
        f"@main = a & @loop ~ ({length} a)",
        "@loop = (?((0 @loop__C0) a) a)",
        "@loop__C0 = a & @loop ~ a",
        "",
    ])


def bitonic_sum(log2n: int, seed: int, seq: int = PCG_DEFAULT_SEQ) -> str:
    """Bitonic sort of 2^log2n seeded keys, then the sum of the sorted keys
    (mod 2^24), so the normal form is one number."""
    keys = pcg_keys(1 << log2n, seed, seq)
    root, defs = _data_tree("K", [str(k) for k in keys])
    lines = [
        f"@main = a & @sum ~ ({log2n} (@sorted a))",
        f"@sorted = a & @sort ~ ({log2n} (0 ({root} a)))",
        "@sum = (?(((a a) @sum__C0) b) b)",
        "@sum__C0 = ({a c} ((b d) f))",
        "  &! @sum ~ (a (b $([+] $(e f))))",
        "  &! @sum ~ (c (d e))",
        BITONIC_DEFS,
    ] + defs
    return "\n".join(lines) + "\n"


def mixed_batch(count: int = 4096, seed: int = 0x4D495845) -> list[tuple[str, dict]]:
    """Per-net programs of the 4096-net mixed batch: 1/3 tree sums with depth
    uniform in 8..18, 1/3 bitonic sorts of 2^6..2^12 keys, 1/3 countdown loops
    of length log-uniform in 10..1e5. Returns [(code, description)]."""
    rng = PCG32(seed, PCG_DEFAULT_SEQ)
    nets = []
    for i in range(count):
        kind = i % 3
        if kind == 0:
            d = 8 + rng.next() % 11
            nets.append((tree_sum(d), {"family": "tree_sum", "depth": d}))
        elif kind == 1:
            k = 6 + rng.next() % 7
            s = rng.next() | (rng.next() << 32)
            nets.append((bitonic_sum(k, s), {"family": "bitonic", "log2n": k, "seed": s}))
        else:
            u = rng.uniform()
            length = int(round(math.exp(math.log(10) + u * (math.log(1e5) - math.log(10)))))
            nets.append((countdown(length), {"family": "countdown", "length": length}))
    return nets


def serving_pool(count: int = 96, seed: int = 0x53525645) -> list[tuple[str, dict]]:
    """Request templates of the serving workload at its stated scale: the
    mixed batch's three families, each net's size log-uniform from 2^8 to
    2^22 nodes -- tree sums of 2^7..2^21 leaves (about twice as many nodes),
    bitonic sums of the most keys n with n log2(n)^2 / 2 within the size
    (2^6..2^14), countdown loops of size/4 steps (10..1e5). Returns
    [(code, description)]."""
    rng = PCG32(seed, PCG_DEFAULT_SEQ)
    nets = []
    for i in range(count):
        kind = i % 3
        lg = 8 + rng.uniform() * 14  # log2 of the size in nodes
        if kind == 0:
            d = min(21, max(7, int(round(lg)) - 1))
            nets.append((tree_sum(d), {"family": "tree_sum", "depth": d, "log2_size": lg}))
        elif kind == 1:
            k = 6
            while k < 14 and (1 << (k + 1)) * (k + 1) ** 2 / 2 <= 2 ** lg:
                k += 1
            s = rng.next() | (rng.next() << 32)
            nets.append((bitonic_sum(k, s), {"family": "bitonic", "log2n": k, "seed": s, "log2_size": lg}))
        else:
            length = int(min(1e5, max(10, round(2 ** lg / 4))))
            nets.append((countdown(length), {"family": "countdown", "length": length, "log2_size": lg}))
    return nets


def poisson_arrivals(count: int, rate: float, seed: int = 0x5E21E) -> list[float]:
    """Arrival times (seconds) of a Poisson process of `rate` requests/s."""
    rng = PCG32(seed, PCG_DEFAULT_SEQ)
    t, out = 0.0, []
    for _ in range(count):
        t += -math.log1p(-rng.uniform()) / rate
        out.append(t)
    return out


def serving_requests(count: int, rate: float, pool: int = 4096, seed: int = 0x5E21E) -> tuple[list[float], list[int]]:
    """`count` requests arriving as a Poisson process of `rate`/s, each a net
    drawn uniformly from the first `pool` nets of mixed_batch (the mixed
    batch's families). Returns (arrival times, template index per request)."""
    rng = PCG32(seed ^ 0xA5A5A5A5, PCG_DEFAULT_SEQ)
    return poisson_arrivals(count, rate, seed), [rng.next() % pool for _ in range(count)]
