"""Generates the golden fixtures of the parity tests (run here, where the
reference sources exist; the fixtures travel, the reference does not).

  reference_programs.json  every non-IO `.hvm` program of the reference's test
                           suite (tests/programs/**, examples/**) with
                           - the snapshot's expected `Result:` line
                             (tests/snapshots/*.snap, produced by `hvm run`),
                           - the `Result:` line and `- ITRS:` count printed
                             by the reference's own C runtime (`hvm run-c`,
                             built in place by oracle/Makefile as
                             oracle/_ref/hvm_ref) on this repository's book
                             buffer.
  batch_mixed_4096.json    per net of the 4096-net mixed batch
                           (workloads.mixed_batch): its family and size, the
                           reference C runtime's interaction count and result.
  serving_pool.json        the same for the serving workload's request
                           templates (workloads.serving_pool: sizes up to
                           2^22 nodes).
  io_programs.json         the reference's IO programs (tests/programs/io,
                           examples/demo_io) run by the reference C runtime
                           in a scratch directory holding the files they
                           open, with the test harness's stdin
                           (tests/run.rs:79-96): printed lines, `Result:`,
                           `- ITRS:`, and the snapshot's text; under "dl",
                           DL_CALL programs calling the test library
                           dl_test.c (the reference binary runs each
                           function's C-runtime twin).
  configs.json             the same two fields for the seeded benchmark
                           workloads (lambdavm-rust_gb300/workloads.py), with
                           large results stored as a SHA-256 of their
                           canonical form, plus the algorithmic bytes of the
                           evaluation counted by the oracle (-w), the
                           roofline numerator.

Usage: python tests/golden/make_golden.py [--reference /root/reference] [--only-io | --only-dl | --only-batch |
                                          --only-serving]
"""
from __future__ import annotations

import argparse
import glob
import hashlib
import importlib
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
H = importlib.import_module("lambdavm-rust_gb300")
W = importlib.import_module("lambdavm-rust_gb300.workloads")
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "hvm_ref")
PORT_BIN = os.path.join(ROOT, "oracle", "_build", "hvm_oracle")


def algorithmic_counts(code: str) -> tuple[int, int]:
    """Word-touch bytes and atomic operations (node takes + var exchanges) of
    the whole evaluation, counted by the oracle (-w)."""
    buf = H.book_from_text(code)
    with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as f:
        buf.tofile(f.name)
        path = f.name
    try:
        r = subprocess.run([PORT_BIN, "-w", path], capture_output=True, text=True, timeout=3600, check=True)
    finally:
        os.unlink(path)
    return (int(re.search(r"^- BYTES: (\d+)$", r.stdout, re.M).group(1)),
            int(re.search(r"^- ATOMICS: (\d+)$", r.stdout, re.M).group(1)))


CONFIG_CASES = {
    "tree_sum_d12": lambda: W.tree_sum(12),
    "tree_sum_d20": lambda: W.tree_sum(20),
    "bitonic_sort_2p8": lambda: W.bitonic_sort(8),
    "bitonic_sort_2p12": lambda: W.bitonic_sort(12),
    "bitonic_sort_2p16": lambda: W.bitonic_sort(16),
    "skewed_fold_2p10": lambda: W.skewed_fold(10),
    "skewed_fold_2p18": lambda: W.skewed_fold(18),
    "countdown_100000": lambda: W.countdown(100000),
}


def config_code(name: str) -> str:
    return CONFIG_CASES[name]()


def refresh_counts() -> None:
    """Recounts the algorithmic bytes and atomics of every entry of
    configs.json (the reference's results in it are left as they are)."""
    path = os.path.join(HERE, "configs.json")
    cfg = json.load(open(path))
    for name, entry in cfg.items():
        entry["algorithmic_bytes"], entry["algorithmic_atomics"] = algorithmic_counts(config_code(name))
        print(name, entry["algorithmic_bytes"], entry["algorithmic_atomics"])
    with open(path, "w") as f:
        json.dump(cfg, f, indent=1)


def run_ref(code: str) -> dict:
    buf = H.book_from_text(code)
    with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as f:
        buf.tofile(f.name)
        path = f.name
    try:
        r = subprocess.run([REF_BIN, path], capture_output=True, text=True, timeout=3600)
    finally:
        os.unlink(path)
    res = re.search(r"^Result: (.*)$", r.stdout, re.M)
    itrs = re.search(r"^- ITRS: (\d+)$", r.stdout, re.M)
    if r.returncode != 0 or not res or not itrs:
        raise RuntimeError(f"reference run failed: rc={r.returncode}\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    return {"result": res.group(1), "itrs": int(itrs.group(1))}


# Files the IO programs open, relative to their working directory: the first
# 47 bytes of LICENSE are what tests/programs/io/basic.hvm prints.
IO_FILES = {"LICENSE": " " * 33 + "Apache License\n" + "".join(f"fixture line {i:05d}\n" for i in range(1500)),
            "README.md": "# readme\n"}
# A larger read: tests/programs/io/basic.hvm with its READ of 47 bytes made 20000.
BIG_READ = ("@call ~ (d ((e 47) f))", "@call ~ (d ((e 20000) f))")
IO_STDIN = "io from the tests\n"


REF_DL_BIN = os.path.join(ROOT, "oracle", "_ref", "hvm_ref_dl")


def run_ref_io(code: str, dl_lib: str | None = None) -> dict:
    buf = H.book_from_text(code)
    with tempfile.TemporaryDirectory() as cwd:
        for name, text in IO_FILES.items():
            with open(os.path.join(cwd, name), "w") as f:
                f.write(text)
        if dl_lib:
            build_dl_lib(os.path.join(cwd, dl_lib))
        path = os.path.join(cwd, "book.bin")
        buf.tofile(path)
        r = subprocess.run([REF_DL_BIN if dl_lib else REF_BIN, path], capture_output=True, text=True, timeout=600,
                           cwd=cwd, input=IO_STDIN)
    res = re.search(r"^Result: (.*)$", r.stdout, re.M)
    itrs = re.search(r"^- ITRS: (\d+)$", r.stdout, re.M)
    if r.returncode != 0 or not res or not itrs:
        raise RuntimeError(f"reference run failed: rc={r.returncode}\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    printed = r.stdout[:res.start()]
    return {"printed": printed, "result": res.group(1), "itrs": int(itrs.group(1))}


def make_io(ref: str) -> None:
    out = []
    files = sorted(glob.glob(os.path.join(ref, "tests", "programs", "io", "*.hvm"))
                   + glob.glob(os.path.join(ref, "examples", "demo_io", "*.hvm")))
    for path in files:
        rel = os.path.relpath(path, ref)
        code = open(path).read()
        key = rel.replace("tests/programs/", "").replace("examples/", "").replace("/", "__")
        snap = os.path.join(ref, "tests", "snapshots", f"run__io_file@{key}.snap")
        snapshot = open(snap).read().split("---\n", 2)[-1] if os.path.exists(snap) else None
        entry = {"name": rel, "code": code, "snapshot": snapshot, **run_ref_io(code)}
        out.append(entry)
        print(rel, entry["itrs"], repr(entry["printed"][:60]))
        if rel.endswith("io/basic.hvm") and BIG_READ[0] in code:
            big = code.replace(BIG_READ[0], BIG_READ[1])
            entry = {"name": rel + " (READ 20000)", "code": big, "snapshot": None, **run_ref_io(big)}
            out.append(entry)
            print(entry["name"], entry["itrs"], len(entry["printed"]))
    with open(os.path.join(HERE, "io_programs.json"), "w") as f:
        json.dump({"files": IO_FILES, "stdin": IO_STDIN, "programs": out}, f, indent=1)


# DL_CALL programs: DL_OPEN the test library (dl_test.c), DL_CALL one of its
# functions on an argument and return the result (run by the reference binary
# built with its functions exported, oracle/Makefile ref-dl). The program around the
# calls is the IO prelude of tests/programs/io/open1.hvm (IO/bind, call, the
# String constructors); each symbol has a C-runtime twin (`*_c`) of the same
# length that the reference binary calls, the `*_g` one is the GPU runtime's.
DL_LIB = "libdltest.so"
DL_CASES = [("inc", 41), ("greet", "abc"), ("nosuch", 0)]  # nosuch: no such symbol in either runtime


def build_dl_lib(out: str) -> None:
    subprocess.run(["gcc", "-O2", "-shared", "-fPIC", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "dl_test.c"), "-o", out], check=True)


def hvm_string(name: str, text: str) -> str:
    if not text:
        return f"@{name} = @String/Nil\n"
    lines = [f"@{name} = k0"]
    for i, ch in enumerate(text):
        tail = f"k{i + 1}" if i + 1 < len(text) else "@String/Nil"
        lines.append(f"  & @String/Cons ~ ({ord(ch)} ({tail} k{i}))")
    return "\n".join(lines) + "\n"


def dl_program(prelude: str, symbol: str, arg) -> str:
    arg_port = str(arg) if isinstance(arg, int) else "@s_arg"
    code = prelude.rstrip() + "\n\n"
    code += "@unwrap = (((* (a a)) b) b)\n\n"
    code += ("@main = s\n  & @IO/bind ~ (o ((((p p) (@dl_step r)) r) s))\n"
             "  & @call ~ (@s_open ((@s_path 0) o))\n\n")
    code += ("@dl_step = (r s)\n  & @unwrap ~ (r h)\n"
             "  & @IO/bind ~ (o ((((p p) (@IO/wrap q)) q) s))\n"
             f"  & @call ~ (@s_call ((h (@s_sym {arg_port})) o))\n\n")
    code += hvm_string("s_open", "DL_OPEN") + hvm_string("s_path", "./" + DL_LIB)
    code += hvm_string("s_call", "DL_CALL") + hvm_string("s_sym", symbol)
    if not isinstance(arg, int):
        code += hvm_string("s_arg", arg)
    return code


def io_prelude(ref: str) -> str:
    text = open(os.path.join(ref, "tests", "programs", "io", "open1.hvm")).read()
    defs = re.split(r"\n(?=@)", text)
    return "\n".join(d.rstrip() + "\n" for d in defs
                     if not d.startswith("@main ") and not d.startswith("@test-io "))


def make_dl(ref: str) -> None:
    path = os.path.join(HERE, "io_programs.json")
    data = json.load(open(path))
    prelude = io_prelude(ref)
    out = []
    for fn, arg in DL_CASES:
        sym_c, sym_g = (fn + "_x", fn + "_x") if fn == "nosuch" else (fn + "_c", fn + "_g")
        code_c = dl_program(prelude, sym_c, arg)
        entry = {"name": f"dl_call {fn}", "code": dl_program(prelude, sym_g, arg), **run_ref_io(code_c, DL_LIB)}
        out.append(entry)
        print(entry["name"], entry["itrs"], entry["result"][:80])
    # two_g has no C twin: its known answer is the inc program's with the Ok
    # payload 42 replaced by the pair (41 42); the payload is never reduced
    # and the symbol names have one length, so the interaction count is the same.
    inc = out[0]
    pair = {"name": "dl_call pair (known answer)", "code": dl_program(prelude, "two_g", 41),
            "printed": inc["printed"], "result": inc["result"].replace("(((0 (42 ", "(((0 ((41 42) ", 1),
            "itrs": inc["itrs"]}
    assert pair["result"] != inc["result"]
    out.append(pair)
    data["dl_lib"] = DL_LIB
    data["dl"] = out
    with open(path, "w") as f:
        json.dump(data, f, indent=1)


def _batch_entry(item):
    idx, code, info = item
    r = run_ref(code)
    return {"net": idx, **info, "itrs": r["itrs"], "result": r["result"]}


def make_batch(count: int = 4096, workers: int = 4) -> None:
    import multiprocessing as mp
    nets = W.mixed_batch(count)
    items = [(i, code, info) for i, (code, info) in enumerate(nets)]
    with mp.get_context("spawn").Pool(workers) as pool:
        out = pool.map(_batch_entry, items, chunksize=8)
    with open(os.path.join(HERE, f"batch_mixed_{count}.json"), "w") as f:
        json.dump({"count": count, "total_itrs": sum(e["itrs"] for e in out), "nets": out}, f)
    print("batch", count, sum(e["itrs"] for e in out))


def make_serving(count: int = 96, workers: int = 4) -> None:
    import multiprocessing as mp
    nets = W.serving_pool(count)
    items = [(i, code, info) for i, (code, info) in enumerate(nets)]
    with mp.get_context("spawn").Pool(workers) as pool:
        out = pool.map(_batch_entry, items, chunksize=1)
    with open(os.path.join(HERE, "serving_pool.json"), "w") as f:
        json.dump({"count": count, "nets": out}, f, indent=0)
    print("serving pool", count, sum(e["itrs"] for e in out))


def snapshot_result(ref: str, rel: str) -> str | None:
    key = rel.replace("tests/programs/", "").replace("examples/", "").replace("/", "__")
    for snap in glob.glob(os.path.join(ref, "tests", "snapshots", "*.snap")):
        if os.path.basename(snap) in (f"run__file@{key}.snap",):
            body = open(snap).read().split("---\n", 2)[-1]
            m = re.search(r"^Result: (.*)$", body, re.M)
            return m.group(1) if m else body.strip()
    return None


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--skip-configs", action="store_true")
    ap.add_argument("--only-batch", action="store_true")
    ap.add_argument("--only-io", action="store_true")
    ap.add_argument("--only-counts", action="store_true")
    ap.add_argument("--only-dl", action="store_true")
    ap.add_argument("--only-serving", action="store_true")
    args = ap.parse_args()
    if args.only_counts:
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle")], check=True)
        refresh_counts()
        return
    if args.only_batch:
        make_batch()
        return
    if args.only_serving:
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "stage", "ref", f"REF_ROOT={args.reference}"], check=True)
        make_serving()
        return
    if args.only_dl:
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "stage", "ref-dl", f"REF_ROOT={args.reference}"],
                       check=True)
        make_dl(args.reference)
        return
    if args.only_io:
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "stage", "ref", f"REF_ROOT={args.reference}"], check=True)
        make_io(args.reference)
        return
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "stage", "ref", f"REF_ROOT={args.reference}"], check=True)
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle")], check=True)

    progs = []
    files = sorted(glob.glob(os.path.join(args.reference, "tests", "programs", "**", "*.hvm"), recursive=True)
                   + glob.glob(os.path.join(args.reference, "examples", "**", "*.hvm"), recursive=True))
    for path in files:
        rel = os.path.relpath(path, args.reference)
        code = open(path).read()
        if "@test-io = 1" in code or "@test-skip = 1" in code or "/io/" in rel or "demo_io" in rel:
            continue  # IO builtins are outside the evaluator path
        entry = {"name": rel, "code": code, "snapshot": snapshot_result(args.reference, rel)}
        try:
            entry.update(run_ref(code))
        except H.HvmError as e:
            entry.update({"build_error": str(e)})
        except RuntimeError as e:
            entry.update({"ref_error": str(e)})
        progs.append(entry)
        print(rel, entry.get("itrs"), entry.get("build_error", ""))
    with open(os.path.join(HERE, "reference_programs.json"), "w") as f:
        json.dump(progs, f, indent=1)

    if args.skip_configs:
        return
    out = {}
    for name in CONFIG_CASES:
        code = config_code(name)
        r = run_ref(code)
        canon = H.canonical(r["result"])
        nbytes, natomics = algorithmic_counts(code)
        entry = {"itrs": r["itrs"], "canonical_sha256": hashlib.sha256(canon.encode()).hexdigest(),
                 "algorithmic_bytes": nbytes, "algorithmic_atomics": natomics}
        if len(r["result"]) <= 4096:
            entry["result"] = r["result"]
        out[name] = entry
        print(name, entry["itrs"])
    with open(os.path.join(HERE, "configs.json"), "w") as f:
        json.dump(out, f, indent=1)
    make_batch()


if __name__ == "__main__":
    main()
