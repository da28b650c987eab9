"""GB300-native HVM2 evaluator: Python host binding.

Mirrors the reference's surface for the `hvm run-cu` path:
  * `book_from_text(code)`  -- `ast::Book::parse(code).build().to_buffer()`
                               (src/ast.rs, src/hvm.rs:957-1003)
  * `hvm_cu(book)`          -- `extern "C" hvm_cu(u32*)` (src/hvm.cu:2320),
                               printing the reference's output lines
  * `Runtime`               -- the re-entrant handle API of include/hvm_gb300.h

Everything computes through `libhvm_gb300.so` (sm_103a CUDA). There is no CPU
fallback: if the library is missing the import of `lib()` raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libhvm_gb300.so")
# The same runtime over 64-bit ports (128-bit node pairs, spaces of up to
# 2^32 words each): Runtime(port64=True).
LIB64_PATH = os.path.join(PKG_DIR, "libhvm_gb300_p64.so")
CLI_PATH = os.path.join(PKG_DIR, "hvm")

_lib = None
_lib64 = None


class HvmError(RuntimeError):
    pass


class Config(ctypes.Structure):
    _fields_ = [
        ("device", ctypes.c_int32),
        ("threads_per_block", ctypes.c_uint32),
        ("stack_cap", ctypes.c_uint32),
        ("blocks_per_sm", ctypes.c_uint32),
        ("node_log2", ctypes.c_uint32),
        ("vars_log2", ctypes.c_uint32),
        ("ring_log2", ctypes.c_uint32),
        ("max_turns", ctypes.c_uint32),
        ("stop_frac_q8", ctypes.c_uint32),
        ("trace_cap", ctypes.c_uint32),
        ("reg_cap_blocks", ctypes.c_uint32),
        ("profile", ctypes.c_uint32),
        ("graph_turns", ctypes.c_uint32),
        ("node_page_log2", ctypes.c_uint32),
        ("var_page_log2", ctypes.c_uint32),
        ("max_pages", ctypes.c_uint32),
        ("steal_min", ctypes.c_uint32),
        ("turn_budget_cap", ctypes.c_uint32),
        ("narrow_below", ctypes.c_uint32),
        ("narrow_reg_cap", ctypes.c_uint32),
        ("rule_select", ctypes.c_uint32),
        ("fast_calls", ctypes.c_uint32),
        ("local_nets", ctypes.c_uint32),
        ("persistent", ctypes.c_uint32),
        ("upper_half", ctypes.c_uint32),
    ]


class Turn(ctypes.Structure):
    _fields_ = [
        ("t_ns", ctypes.c_uint64),
        ("live_nodes", ctypes.c_int64),
        ("itrs", ctypes.c_uint64),
        ("pending", ctypes.c_uint64),
        ("dry", ctypes.c_uint32),
        ("stopped", ctypes.c_uint32),
        ("budget", ctypes.c_uint32),
        ("per_thread", ctypes.c_uint32),
        ("features", ctypes.c_float * 16),
        ("outputs", ctypes.c_float * 3),
    ]


class _Stats(ctypes.Structure):
    _fields_ = [
        ("itrs", ctypes.c_uint64),
        ("leak", ctypes.c_uint64),
        ("turns", ctypes.c_uint64),
        ("retries", ctypes.c_uint64),
        ("rule_hist", ctypes.c_uint64 * 8),
        ("prof", ctypes.c_uint64 * 8),
        ("seconds", ctypes.c_double),
        ("kernel_ms", ctypes.c_double),
        ("turn_launches", ctypes.c_uint64),
        ("launches", ctypes.c_uint64),
        ("h2d_bytes", ctypes.c_uint64),
        ("d2h_bytes", ctypes.c_uint64),
        ("threads", ctypes.c_uint32),
        ("grid", ctypes.c_uint32),
        ("block", ctypes.c_uint32),
    ]


# Turn scheduler modes and the MLP's shape (include/hvm_gb300.h).
POLICY_FIXED, POLICY_LEARNED, POLICY_CONSTANT, POLICY_SCRIPT = 0, 1, 2, 3
POLICY_IN, POLICY_HID, POLICY_OUT = 16, 64, 3
POLICY_PARAMS = POLICY_HID * POLICY_IN + POLICY_HID + POLICY_HID * POLICY_HID + POLICY_HID + POLICY_OUT * POLICY_HID + POLICY_OUT


RULE_NAMES = ("LINK", "CALL", "VOID", "ERAS", "ANNI", "COMM", "OPER", "SWIT")

# Every symbol include/hvm_gb300.h declares.
EXPORTED_SYMBOLS = (
    "hvm_cu",
    "hvm_gb300_book_from_text",
    "hvm_gb300_canonical_tree",
    "hvm_gb300_compile_calls",
    "hvm_gb300_default_config",
    "hvm_gb300_create",
    "hvm_gb300_load_book",
    "hvm_gb300_run",
    "hvm_gb300_result",
    "hvm_gb300_trace",
    "hvm_gb300_reset_counters",
    "hvm_gb300_run_noalloc",
    "hvm_gb300_load_batch",
    "hvm_gb300_run_batch",
    "hvm_gb300_batch_roots",
    "hvm_gb300_run_stream",
    "hvm_gb300_set_requests",
    "hvm_gb300_batch_result",
    "hvm_gb300_count_live",
    "hvm_gb300_set_policy",
    "hvm_gb300_policy_forward",
    "hvm_gb300_policy_grad",
    "hvm_gb300_policy_train",
    "hvm_gb300_atomic_peak",
    "hvm_gb300_io_expand",
    "hvm_gb300_io_node_load",
    "hvm_gb300_io_make_node",
    "hvm_gb300_io_readback_tup",
    "hvm_gb300_io_readback_bytes",
    "hvm_gb300_io_inject_bytes",
    "hvm_gb300_wait_probe",
    "hvm_gb300_error",
    "hvm_gb300_destroy",
)


def lib() -> ctypes.CDLL:
    """Loads libhvm_gb300.so (built in-tree by build.py); raises if absent."""
    global _lib
    if _lib is None:
        _lib = _load(LIB_PATH)
    return _lib


def lib64() -> ctypes.CDLL:
    """Loads libhvm_gb300_p64.so, the 64-bit port build; raises if absent."""
    global _lib64
    if _lib64 is None:
        _lib64 = _load(LIB64_PATH)
    return _lib64


def _load(path: str) -> ctypes.CDLL:
    if not os.path.exists(path):
        raise HvmError(f"{path} is missing: build it with `python lambdavm-rust_gb300/build.py` "
                       "or `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(path)
    u32p = ctypes.POINTER(ctypes.c_uint32)
    L.hvm_cu.argtypes = [u32p]
    L.hvm_cu.restype = None
    L.hvm_gb300_book_from_text.argtypes = [ctypes.c_char_p, u32p, ctypes.c_size_t,
                                           ctypes.POINTER(ctypes.c_size_t), ctypes.c_char_p, ctypes.c_size_t]
    L.hvm_gb300_canonical_tree.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t,
                                           ctypes.POINTER(ctypes.c_size_t), ctypes.c_char_p, ctypes.c_size_t]
    L.hvm_gb300_compile_calls.argtypes = [u32p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t,
                                          ctypes.POINTER(ctypes.c_size_t), ctypes.c_char_p, ctypes.c_size_t]
    L.hvm_gb300_default_config.argtypes = [ctypes.POINTER(Config)]
    L.hvm_gb300_wait_probe.argtypes = [ctypes.c_int32, ctypes.c_uint32, u32p, ctypes.POINTER(ctypes.c_double)]
    L.hvm_gb300_default_config.restype = None
    L.hvm_gb300_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(ctypes.c_void_p)]
    L.hvm_gb300_load_book.argtypes = [ctypes.c_void_p, u32p, ctypes.c_size_t]
    L.hvm_gb300_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Stats)]
    L.hvm_gb300_result.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t,
                                   ctypes.POINTER(ctypes.c_size_t)]
    L.hvm_gb300_trace.argtypes = [ctypes.c_void_p, ctypes.POINTER(Turn), ctypes.c_size_t,
                                  ctypes.POINTER(ctypes.c_size_t)]
    L.hvm_gb300_run_noalloc.argtypes = [u32p, ctypes.c_size_t, u32p, u32p, ctypes.c_size_t,
                                        ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_uint64),
                                        ctypes.c_char_p, ctypes.c_size_t]
    L.hvm_gb300_load_batch.argtypes = [ctypes.c_void_p, ctypes.POINTER(u32p), ctypes.POINTER(ctypes.c_size_t),
                                       ctypes.c_uint32]
    L.hvm_gb300_run_batch.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Stats)]
    L.hvm_gb300_batch_roots.argtypes = [ctypes.c_void_p, u32p, ctypes.c_size_t]
    L.hvm_gb300_set_requests.argtypes = [ctypes.c_void_p, u32p, ctypes.c_uint32]
    L.hvm_gb300_run_stream.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_uint32,
                                       ctypes.c_double, ctypes.c_uint32, ctypes.POINTER(ctypes.c_double), u32p,
                                       ctypes.POINTER(_Stats)]
    L.hvm_gb300_batch_result.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_size_t,
                                         ctypes.POINTER(ctypes.c_size_t)]
    L.hvm_gb300_count_live.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
    fp = ctypes.POINTER(ctypes.c_float)
    L.hvm_gb300_set_policy.argtypes = [ctypes.c_void_p, ctypes.c_uint32, fp, ctypes.c_size_t, fp]
    L.hvm_gb300_policy_forward.argtypes = [ctypes.c_int, fp, fp, ctypes.c_size_t, fp, ctypes.c_char_p,
                                           ctypes.c_size_t]
    L.hvm_gb300_policy_grad.argtypes = [ctypes.c_int, fp, fp, fp, fp, ctypes.c_size_t, fp, fp, ctypes.c_char_p,
                                        ctypes.c_size_t]
    L.hvm_gb300_policy_train.argtypes = [ctypes.c_int, fp, fp, fp, fp, ctypes.c_size_t, ctypes.c_uint32,
                                         ctypes.c_float, fp, ctypes.c_char_p, ctypes.c_size_t]
    L.hvm_gb300_atomic_peak.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double),
                                        ctypes.c_char_p, ctypes.c_size_t]
    L.hvm_gb300_reset_counters.argtypes = [ctypes.c_void_p]
    L.hvm_gb300_reset_counters.restype = None
    L.hvm_gb300_error.argtypes = [ctypes.c_void_p]
    L.hvm_gb300_error.restype = ctypes.c_char_p
    L.hvm_gb300_destroy.argtypes = [ctypes.c_void_p]
    L.hvm_gb300_destroy.restype = None
    return L


def book_from_text(code: str) -> np.ndarray:
    """Parses `.hvm` text into the reference's u32 book buffer."""
    L = lib()
    n = ctypes.c_size_t()
    err = ctypes.create_string_buffer(4096)
    data = code.encode()
    rc = L.hvm_gb300_book_from_text(data, None, 0, ctypes.byref(n), err, len(err))
    if rc:
        raise HvmError(err.value.decode())
    buf = np.zeros(n.value, dtype=np.uint32)
    rc = L.hvm_gb300_book_from_text(data, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                    n.value, ctypes.byref(n), err, len(err))
    if rc:
        raise HvmError(err.value.decode())
    return buf


def canonical(tree_text: str) -> str:
    """Canonical form of a printed tree: vars renamed by first occurrence,
    numbers as 29-bit words (bit-exact comparison, f24 included)."""
    L = lib()
    n = ctypes.c_size_t()
    err = ctypes.create_string_buffer(4096)
    data = tree_text.encode()
    rc = L.hvm_gb300_canonical_tree(data, None, 0, ctypes.byref(n), err, len(err))
    if rc:
        raise HvmError(err.value.decode())
    out = ctypes.create_string_buffer(n.value + 1)
    rc = L.hvm_gb300_canonical_tree(data, out, n.value + 1, ctypes.byref(n), err, len(err))
    if rc:
        raise HvmError(err.value.decode())
    return out.value.decode()


def compile_calls(book) -> str:
    """CUDA source of the compiled calls for a book (text or serialized
    words): what `hvm gen-cu --compiled` appends to the standalone program."""
    L = lib()
    words = book_from_text(book) if isinstance(book, str) else np.ascontiguousarray(book, dtype=np.uint32)
    ptr = words.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    n = ctypes.c_size_t()
    err = ctypes.create_string_buffer(4096)
    if L.hvm_gb300_compile_calls(ptr, words.size, None, 0, ctypes.byref(n), err, len(err)):
        raise HvmError(err.value.decode())
    out = ctypes.create_string_buffer(n.value + 1)
    if L.hvm_gb300_compile_calls(ptr, words.size, out, n.value + 1, ctypes.byref(n), err, len(err)):
        raise HvmError(err.value.decode())
    return out.value.decode()


@dataclass
class RunStats:
    itrs: int
    leak: int
    turns: int
    retries: int
    seconds: float
    threads: int
    grid: int
    block: int
    rule_hist: dict = field(default_factory=dict)
    prof: tuple = ()
    kernel_ms: float = 0.0
    turn_launches: int = 0
    launches: int = 0
    h2d_bytes: int = 0
    d2h_bytes: int = 0

    @property
    def mips(self) -> float:
        return self.itrs / self.seconds / 1e6 if self.seconds > 0 else float("nan")


class Runtime:
    """One GPU net (include/hvm_gb300.h handle API)."""

    def __init__(self, device: int = 0, port64: bool = False, **overrides):
        L = lib64() if port64 else lib()
        self._L = L
        cfg = Config()
        L.hvm_gb300_default_config(ctypes.byref(cfg))
        cfg.device = device
        for k, v in overrides.items():
            if not hasattr(cfg, k):
                raise TypeError(f"unknown config field {k}")
            setattr(cfg, k, v)
        self.config = cfg
        h = ctypes.c_void_p()
        rc = L.hvm_gb300_create(ctypes.byref(cfg), ctypes.byref(h))
        self._h = h
        if rc:
            msg = L.hvm_gb300_error(h).decode() if h else "create failed"
            self.close()
            raise HvmError(msg)

    def _check(self, rc: int) -> None:
        if rc:
            raise HvmError(self._L.hvm_gb300_error(self._h).decode())

    def load(self, book) -> None:
        if isinstance(book, str):
            book = book_from_text(book)
        buf = np.ascontiguousarray(np.asarray(book, dtype=np.uint32))
        self._book = buf
        self._check(self._L.hvm_gb300_load_book(self._h, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                              buf.size))

    def run(self) -> RunStats:
        st = _Stats()
        self._check(self._L.hvm_gb300_run(self._h, ctypes.byref(st)))
        return self._stats(st)

    @staticmethod
    def _stats(st) -> RunStats:
        return RunStats(itrs=st.itrs, leak=st.leak, turns=st.turns, retries=st.retries, seconds=st.seconds,
                        threads=st.threads, grid=st.grid, block=st.block,
                        rule_hist={RULE_NAMES[i]: int(st.rule_hist[i]) for i in range(8)},
                        prof=tuple(int(x) for x in st.prof), kernel_ms=st.kernel_ms,
                        turn_launches=st.turn_launches, launches=st.launches,
                        h2d_bytes=st.h2d_bytes, d2h_bytes=st.d2h_bytes)

    def load_batch(self, books) -> None:
        """Loads independent nets (book buffers or .hvm texts) as one batch."""
        bufs = [np.ascontiguousarray(np.asarray(book_from_text(b) if isinstance(b, str) else b, dtype=np.uint32))
                for b in books]
        self._batch = bufs
        u32p = ctypes.POINTER(ctypes.c_uint32)
        ptrs = (u32p * len(bufs))(*[b.ctypes.data_as(u32p) for b in bufs])
        sizes = (ctypes.c_size_t * len(bufs))(*[b.size for b in bufs])
        self._check(self._L.hvm_gb300_load_batch(self._h, ptrs, sizes, len(bufs)))

    def run_batch(self) -> RunStats:
        st = _Stats()
        self._check(self._L.hvm_gb300_run_batch(self._h, ctypes.byref(st)))
        return self._stats(st)

    def set_requests(self, templates) -> None:
        """Makes request r a copy of loaded net templates[r] (serving)."""
        t = np.ascontiguousarray(templates, dtype=np.uint32)
        self._check(self._L.hvm_gb300_set_requests(self._h, t.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), t.size))
        self._batch = [None] * t.size

    def run_stream(self, arrival_s=None, max_inflight: int = 0, live_frac: float = 0.25, order: int = 0):
        """Continuous batching over the loaded batch; returns (stats, done_s, result_ports)."""
        n = len(self._batch)
        arr = np.zeros(n, dtype=np.float64) if arrival_s is None else np.ascontiguousarray(arrival_s, dtype=np.float64)
        done = np.zeros(n, dtype=np.float64)
        res = np.zeros(n, dtype=np.uint32)
        st = _Stats()
        self._check(self._L.hvm_gb300_run_stream(self._h, arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                               max_inflight, live_frac, order,
                                               done.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                               res.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                               ctypes.byref(st)))
        return self._stats(st), done, res

    def batch_roots(self) -> np.ndarray:
        out = np.zeros(len(self._batch), dtype=np.uint32)
        self._check(self._L.hvm_gb300_batch_roots(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                                out.size))
        return out

    def batch_result(self, net: int) -> str:
        n = ctypes.c_size_t()
        self._check(self._L.hvm_gb300_batch_result(self._h, net, None, 0, ctypes.byref(n)))
        out = ctypes.create_string_buffer(n.value + 1)
        self._check(self._L.hvm_gb300_batch_result(self._h, net, out, n.value + 1, ctypes.byref(n)))
        return out.value.decode()

    def result(self) -> str:
        n = ctypes.c_size_t()
        self._check(self._L.hvm_gb300_result(self._h, None, 0, ctypes.byref(n)))
        out = ctypes.create_string_buffer(n.value + 1)
        self._check(self._L.hvm_gb300_result(self._h, out, n.value + 1, ctypes.byref(n)))
        return out.value.decode()

    def count_live(self) -> dict:
        out = (ctypes.c_uint64 * 5)()
        self._check(self._L.hvm_gb300_count_live(self._h, out))
        return {"nodes": out[0], "vars": out[1], "marked": out[2], "node_pages": out[3], "var_pages": out[4]}

    def reset_counters(self) -> None:
        self._L.hvm_gb300_reset_counters(self._h)

    def trace(self) -> list[dict]:
        """Per-turn records of the last run (needs trace_cap > 0)."""
        n = ctypes.c_size_t()
        self._check(self._L.hvm_gb300_trace(self._h, None, 0, ctypes.byref(n)))
        arr = (Turn * max(1, n.value))()
        self._check(self._L.hvm_gb300_trace(self._h, arr, n.value, ctypes.byref(n)))
        out = []
        for i in range(n.value):
            r = {k: getattr(arr[i], k) for k, _ in Turn._fields_}
            r["features"] = list(r["features"])
            r["outputs"] = list(r["outputs"])
            out.append(r)
        return out

    def set_policy(self, mode: int = POLICY_FIXED, weights=None, constants=None) -> None:
        """Selects the turn scheduler for later runs: POLICY_FIXED, POLICY_LEARNED
        with `weights` (POLICY_PARAMS floats), or POLICY_CONSTANT with 6
        `constants` (budget, stop fraction, static share while fewer redexes
        than threads are pending, then the same three otherwise; -1 keeps the
        fixed policy's choice), or POLICY_SCRIPT with `weights` = 3 floats per
        turn (the decision at the close of turn k; -1 or later turns: fixed)."""
        w = _floats(weights) if weights is not None else None
        c = _floats(constants) if constants is not None else None
        self._check(self._L.hvm_gb300_set_policy(self._h, mode, w, len(w) if w is not None else 0, c))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.hvm_gb300_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _floats(values):
    vals = [float(v) for v in values]
    return (ctypes.c_float * max(1, len(vals)))(*vals) if vals else None


def _float_buf(arr, rows: int, cols: int):
    import numpy as np
    a = np.ascontiguousarray(np.asarray(arr, dtype=np.float32).reshape(rows, cols))
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _err_buf():
    return ctypes.create_string_buffer(512)


def policy_forward(weights, x, device: int = 0):
    """Outputs of the scheduler MLP for each row of `x` (n x 16), computed by
    the routine the turn kernel runs."""
    import numpy as np
    x = np.asarray(x, dtype=np.float32)
    n = x.shape[0]
    w, wp = _float_buf(weights, 1, POLICY_PARAMS)
    xa, xp = _float_buf(x, n, POLICY_IN)
    y = np.zeros((n, POLICY_OUT), dtype=np.float32)
    err = _err_buf()
    if lib().hvm_gb300_policy_forward(device, wp, xp, n, y.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), err, 512):
        raise HvmError(err.value.decode())
    return y


def policy_grad(weights, x, t, sw, device: int = 0):
    """(loss, gradient) of the weighted squared error of the MLP's outputs."""
    import numpy as np
    n = np.asarray(x).shape[0]
    w, wp = _float_buf(weights, 1, POLICY_PARAMS)
    xa, xp = _float_buf(x, n, POLICY_IN)
    ta, tp = _float_buf(t, n, POLICY_OUT)
    sa, sp = _float_buf(sw, n, 1)
    g = np.zeros(POLICY_PARAMS, dtype=np.float32)
    loss = ctypes.c_float()
    err = _err_buf()
    if lib().hvm_gb300_policy_grad(device, wp, xp, tp, sp, n, g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                   ctypes.byref(loss), err, 512):
        raise HvmError(err.value.decode())
    return loss.value, g


def policy_train(weights, x, t, sw, epochs: int, lr: float = 1e-3, device: int = 0):
    """Full-batch Adam training on the GPU; returns (new weights, loss)."""
    import numpy as np
    n = np.asarray(x).shape[0]
    w = np.ascontiguousarray(np.asarray(weights, dtype=np.float32).reshape(POLICY_PARAMS).copy())
    xa, xp = _float_buf(x, n, POLICY_IN)
    ta, tp = _float_buf(t, n, POLICY_OUT)
    sa, sp = _float_buf(sw, n, 1)
    loss = ctypes.c_float()
    err = _err_buf()
    if lib().hvm_gb300_policy_train(device, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), xp, tp, sp, n,
                                    epochs, lr, ctypes.byref(loss), err, 512):
        raise HvmError(err.value.decode())
    return w, loss.value


def atomic_peak(region_words: int = 1 << 24, device: int = 0) -> float:
    """Measured 32-bit atomicExch operations per second at random addresses
    of a region of `region_words` words (the atomic roofline's denominator)."""
    v = ctypes.c_double()
    err = _err_buf()
    if lib().hvm_gb300_atomic_peak(device, region_words, ctypes.byref(v), err, 512):
        raise HvmError(err.value.decode())
    return v.value


def wait_probe(limit_ms: int = 100, device: int = 0) -> tuple[bool, float]:
    """Runs the persistent launches' bounded wait on a word nothing writes:
    (whether the limit ran out, milliseconds waited)."""
    out = ctypes.c_uint32()
    ms = ctypes.c_double()
    if lib().hvm_gb300_wait_probe(device, limit_ms, ctypes.byref(out), ctypes.byref(ms)):
        raise HvmError("wait probe failed")
    return bool(out.value), ms.value


def run_text(code: str, device: int = 0, **cfg) -> tuple[str, RunStats]:
    """Parses, loads and normalises `code`; returns (result tree text, stats)."""
    with Runtime(device=device, **cfg) as rt:
        rt.load(code)
        st = rt.run()
        return rt.result(), st
