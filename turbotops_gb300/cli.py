"""``python -m turbotops_gb300 run <input> [options]`` — the ``turbotops run`` CLI
(src/turbotops.cpp:30-80, :784-935) on the GB300 front end.

Same input formats (text: one point per line, commas/spaces/tabs/semicolons,
'#' comments, UTF-8 BOM stripped; .bin: raw little-endian float32 with
--dim), same options for this path, same output (one bar per line,
'dim birth death' with %.9g, 'inf' for essential classes, canonical order),
same failure convention ('turbotops: <message>' on stderr, exit code 2).
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

USAGE = """usage:
  python -m turbotops_gb300 run <input> [options]   compute a persistence diagram
  python -m turbotops_gb300 --version               print the version and exit

input (run):
  text   one point per line, coordinates separated by commas or spaces ('#' starts a comment)
  .bin   raw little-endian float32, row-major; requires --dim

options:
  --maxdim D          highest homology dimension (default 1)
  --threshold T       filtration cutoff, inclusive (default inf)
  --metric M          l1 | l2 | linf | lp:<p>, p >= 1 (default l2)
  --graph full|knn    complex: all pairs, or the kNN graph (default full)
  -k N                neighbors for --graph knn (default 15)
  --dim D             coordinates per point for .bin input
  --edges             input is a weighted edge list 'i j w' (0-based), one per line
  --mode M            boundary | coboundary | auto (diagrams never depend on it)
  --coboundary, --boundary, --no-coboundary, --engine E   accepted, as --mode
  --threads N         accepted (results never depend on it)
  --memory-budget B   bytes, with optional k/m/g suffix (default: half of RAM); a dense
                      complex whose distance matrix exceeds it is refused, as the reference does
  --output FILE       write the diagram to FILE instead of stdout
  --quiet             no summary on stderr
"""


class CliError(Exception):
    pass


_strtof = None


def _parse_f32(tok: str, what: str) -> float:
    """The host C library's strtof over the whole token, as the reference's
    parse_f32 does (src/turbotops.cpp:119-124): one rounding from the decimal
    (or hexadecimal) text to float32, 'inf'/'nan' spellings accepted, trailing
    characters an error."""
    global _strtof
    if _strtof is None:
        import ctypes
        libc = ctypes.CDLL(None)
        _strtof = libc.strtof
        _strtof.restype = ctypes.c_float
        _strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]
    import ctypes
    raw = tok.encode("utf-8", "surrogateescape")
    buf = ctypes.create_string_buffer(raw)
    end = ctypes.c_void_p()
    v = _strtof(ctypes.cast(buf, ctypes.c_char_p), ctypes.byref(end))
    if not raw or end.value is None or end.value - ctypes.addressof(buf) != len(raw):
        raise CliError(f"bad {what} '{tok}'")
    return float(v)


def _parse_bytes(tok: str) -> int:
    """The reference's parse_bytes (src/turbotops.cpp:86-100): the C library's
    strtod, then, if anything follows the number, its first character must
    be k, m or g (either case: KiB, MiB, GiB); the product must be positive
    and is truncated to whole bytes."""
    import ctypes
    libc = ctypes.CDLL(None)
    strtod = libc.strtod
    strtod.restype = ctypes.c_double
    strtod.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]
    raw = tok.encode("utf-8", "surrogateescape")
    buf = ctypes.create_string_buffer(raw)
    end = ctypes.c_void_p()
    v = strtod(ctypes.cast(buf, ctypes.c_char_p), ctypes.byref(end))
    at = (end.value or ctypes.addressof(buf)) - ctypes.addressof(buf)
    mul = 1.0
    if at < len(raw):
        mul = {ord("k"): 1024.0, ord("m"): 1024.0 ** 2, ord("g"): 1024.0 ** 3}.get(raw[at] | 0x20)
        if mul is None:
            raise CliError(f"bad byte count '{tok}'")
    if not v > 0:
        raise CliError(f"bad byte count '{tok}'")
    b = v * mul
    return (1 << 64) - 1 if b >= 2.0 ** 64 else int(b)


def _parse_u32(tok: str, what: str) -> int:
    if not tok.isdigit():
        raise CliError(f"bad {what} '{tok}'")
    v = int(tok)
    if v > 0xFFFFFFFF:
        raise CliError(f"bad {what} '{tok}' (out of range)")
    return v


def read_text_points(path: str) -> np.ndarray:
    """read_text_points (src/turbotops.cpp:126-155), converted on the GPU
    (tt_parse_points_h): the same lines, comments, separators, strtof values
    and messages."""
    try:
        raw = open(path, "rb").read()
    except OSError:
        raise CliError(f"cannot open {path}") from None
    import ctypes
    from . import api, capi
    ctx = api._context(0)
    cap = len(raw) // 2 + 2
    pts = np.empty(cap, dtype=np.float32)
    n, dim = ctypes.c_uint32(), ctypes.c_uint32()
    st = ctx.L.tt_parse_points_h(ctx.h, raw, len(raw), pts.ctypes.data, cap, ctypes.byref(n), ctypes.byref(dim))
    if st != capi.OK:
        msg = ctx.L.tt_last_error(ctx.h).decode("utf-8", "surrogateescape")
        if st == capi.ERR_INVALID:
            raise CliError(f"{path}: {msg}" if msg.startswith("inconsistent row length") else msg)
        capi.raise_for(st, msg)
    return pts[: n.value * dim.value].reshape(n.value, dim.value).copy()


def _parse_u64(tok: str, what: str) -> int:
    """strtoull, base 10, whole token (src/turbotops.cpp:102-108): an optional
    sign, '-' wrapping modulo 2^64; out of range is an error."""
    body = tok[1:] if tok[:1] in "+-" else tok
    if not body.isdigit():
        raise CliError(f"bad {what} '{tok}'")
    v = int(body)
    if v > 0xFFFFFFFFFFFFFFFF:
        raise CliError(f"bad {what} '{tok}'")
    return (-v) % (1 << 64) if tok[:1] == "-" else v


def read_edges(path: str):
    """A weighted edge list 'i j w' (0-based), one per line (src/turbotops.cpp:173-205):
    '#' comments, ',' and tabs as separators, self loops dropped, both
    directions kept, the smallest weight of a repeated edge."""
    from .api import symmetric_rows
    try:
        lines = open(path, "r", encoding="utf-8", errors="replace").read().split("\n")
    except OSError:
        raise CliError(f"cannot open {path}") from None
    ii, jj, ww = [], [], []
    n = 0
    for lineno, line in enumerate(lines, 1):
        line = line.split("#", 1)[0].replace(",", " ").replace("\t", " ")
        toks = line.split()
        if not toks:
            continue
        if len(toks) < 3:
            raise CliError(f"{path}:{lineno}: expected 'i j w'")
        i = _parse_u64(toks[0], "vertex")
        j = _parse_u64(toks[1], "vertex")
        d = _parse_f32(toks[2], "weight")
        if i == j:
            continue
        if not (d >= 0) or not math.isfinite(d):
            raise CliError(f"{path}:{lineno}: bad weight")
        if max(i, j) >= 0xFFFFFFFF:
            raise CliError("vertex id too large")
        n = max(n, max(i, j) + 1)
        ii.append(i)
        jj.append(j)
        ww.append(d)
    rp, ci, w = symmetric_rows(np.array(ii, np.int64), np.array(jj, np.int64), np.array(ww, np.float32), n)
    return rp, ci, w, n


def read_bin_points(path: str, dim: int) -> np.ndarray:
    if not dim:
        raise CliError("--dim is required for .bin input")
    try:
        raw = np.fromfile(path, dtype="<f4")
    except OSError:
        raise CliError(f"cannot open {path}") from None
    if raw.size % dim:
        raise CliError(f"{path}: size is not a multiple of 4 * dim")
    return raw.reshape(-1, dim).astype(np.float32)


def run(argv: list[str]) -> int:
    from . import api
    if not argv:
        raise CliError("run: missing <input>\n" + USAGE)
    path = argv[0]
    o = {"maxdim": 1, "threshold": math.inf, "metric": "l2", "graph": "full", "k": 15, "dim": 0,
         "output": None, "quiet": False, "edges": False, "memory_budget": 0}
    it = iter(argv[1:])
    for a in it:
        def val():
            try:
                return next(it)
            except StopIteration:
                raise CliError(f"{a} needs a value") from None
        if a == "--maxdim":
            o["maxdim"] = _parse_u32(val(), "maxdim")
        elif a == "--threshold":
            v = val()
            o["threshold"] = math.inf if v == "inf" else _parse_f32(v, "threshold")
        elif a == "--metric":
            o["metric"] = val()
        elif a == "--graph":
            g = val()
            if g not in ("full", "knn"):
                raise CliError("--graph must be full or knn")
            o["graph"] = g
        elif a == "-k":
            o["k"] = _parse_u32(val(), "k")
        elif a == "--dim":
            o["dim"] = _parse_u32(val(), "dim")
        elif a in ("--mode", "--engine"):
            m = val()
            ok = ("auto", "boundary", "coboundary") if a == "--mode" else ("auto", "reducer", "redzed")
            if m not in ok:
                raise CliError(("mode must be auto, boundary or coboundary" if a == "--mode"
                                else "engine must be auto, reducer or redzed"))
        elif a in ("--coboundary", "--boundary", "--no-coboundary", "--quiet"):
            if a == "--quiet":
                o["quiet"] = True
        elif a == "--threads":
            _parse_u32(val(), "threads")
        elif a == "--memory-budget":
            o["memory_budget"] = _parse_bytes(val())
        elif a == "--output":
            o["output"] = val()
        elif a == "--edges":
            o["edges"] = True
        elif a == "--approximate":
            raise CliError(f"{a} is not offered by the GPU front end")
        else:
            raise CliError(f"unknown option '{a}'")
    out_f = None
    if o["output"]:
        try:
            out_f = open(o["output"], "w")
        except OSError:
            raise CliError(f"cannot open {o['output']} for writing") from None
    try:
        if o["edges"]:
            rp, ci, w, nv = read_edges(path)
            if not nv:
                raise CliError(f"{path}: no vertices (empty edge list?)")
            x = None
            dgms, info = api.persistence_graph(rp, ci, w, nv, maxdim=o["maxdim"], threshold=o["threshold"])
        else:
            x = read_bin_points(path, o["dim"]) if path.endswith(".bin") else read_text_points(path)
            dgms, info = api.persistence(x, maxdim=o["maxdim"], threshold=o["threshold"], metric=o["metric"],
                                         graph=o["graph"], k=o["k"], memory_budget=o["memory_budget"])
    except (ValueError, OverflowError, MemoryError) as e:
        raise CliError(str(e)) from None
    text = api.format_diagram(dgms)
    (out_f or sys.stdout).write(text)
    if out_f:
        out_f.close()
    if not o["quiet"]:
        if x is None:
            sys.stderr.write(f"turbotops: graph with {nv} vertices, method {info['method']}, "
                             f"threshold {info['threshold']:.9g}, {info['edges']} edges, "
                             f"{info['seconds_total']:.3f} s\n")
        else:
            n, d = x.shape if x.size else (0, 0)
            sys.stderr.write(f"turbotops: {n} points in R^{d}, method {info['method']}, "
                             f"threshold {info['threshold']:.9g}, {info['edges']} edges, "
                             f"{info['seconds_total']:.3f} s\n")
        for dd, g in enumerate(dgms):
            sys.stderr.write(f"  H{dd}: {len(g)} bars\n")
    return 0


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    try:
        if not argv:
            raise CliError("usage\n" + USAGE)
        if argv[0] in ("--version", "version"):
            print("turbotops 0.1.0 (gb300)")
            return 0
        if argv[0] in ("--help", "help", "-h"):
            print(USAGE)
            return 0
        if argv[0] == "run":
            return run(argv[1:])
        raise CliError(f"unknown command '{argv[0]}'\n" + USAGE)
    except (CliError, RuntimeError, MemoryError, OverflowError, ValueError) as e:
        # the reference's CLI: every std::exception -> "turbotops: <what>", exit 2
        sys.stderr.write(f"turbotops: {e}\n")
        return 2


if __name__ == "__main__":
    sys.exit(main())
