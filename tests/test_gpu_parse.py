"""Text ingestion on the device (tt_parse_points_h) against the reference's
read_text_points (src/turbotops.cpp:126-155) restated below with the host C
library's strtof: every value bit for bit, the same points, the same first
error. Tokens cover the decimal conversion's hard cases: exact halfway
points between adjacent floats (and the nearest decimals above and below
them), subnormals, overflow, more than 19 significant digits, and the
spellings only the host converts (hexadecimal floats, NaN)."""
from __future__ import annotations

import ctypes
import random
from decimal import Decimal, getcontext

import numpy as np
import pytest

from gpu_util import ctx

pytestmark = pytest.mark.gpu

_libc = ctypes.CDLL(None)
_strtof = _libc.strtof
_strtof.restype = ctypes.c_float
_strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]


def strtof_bits(tok: bytes) -> tuple[int, bool]:
    """The value bits std::strtof gives the whole token, and whether it
    consumed all of it (the reference's parse_f32)."""
    buf = ctypes.create_string_buffer(tok)
    end = ctypes.c_char_p()
    v = _strtof(buf, ctypes.byref(end))
    consumed = ctypes.cast(end, ctypes.c_void_p).value - ctypes.addressof(buf)
    ok = len(tok) > 0 and consumed == len(tok)
    return int(np.float32(v).view(np.uint32)), ok


def reference_read(raw: bytes):
    """read_text_points restated: getline on '\\n', cut at '#', ',', '\\t' and
    ';' to spaces, tokens at C white space, strtof over each whole token.
    Returns (bits n x dim) or the error message."""
    if raw[:3] == b"\xef\xbb\xbf":
        raw = raw[3:]
    lines = raw.split(b"\n")
    if lines and lines[-1] == b"":
        lines.pop()
    rows, dim = [], 0
    for line in lines:
        line = line.split(b"#", 1)[0]
        for ch in b",\t;":
            line = line.replace(bytes([ch]), b" ")
        toks = line.split()   # bytes.split() splits at the C locale's white space
        vals = []
        for t in toks:
            b, ok = strtof_bits(t)
            if not ok:
                return f"bad coordinate '{t.decode('latin-1')}'"
            vals.append(b)
        if not vals:
            continue
        if not dim:
            dim = len(vals)
        elif len(vals) != dim:
            return f"inconsistent row length at point {len(rows)}"
        rows.append(vals)
    return np.array(rows, dtype=np.uint32).reshape(len(rows), dim if rows else 0)


def device_read(raw: bytes):
    c = ctx()
    cap = len(raw) // 2 + 2
    pts = np.empty(cap, dtype=np.float32)
    n, dim = ctypes.c_uint32(), ctypes.c_uint32()
    st = c.L.tt_parse_points_h(c.h, raw, len(raw), pts.ctypes.data, cap, ctypes.byref(n), ctypes.byref(dim))
    if st:
        return c.L.tt_last_error(c.h).decode("latin-1")
    return pts[: n.value * dim.value].view(np.uint32).reshape(n.value, dim.value)


def same(raw: bytes):
    want, got = reference_read(raw), device_read(raw)
    if isinstance(want, str) or isinstance(got, str):
        assert got == want
    else:
        assert got.shape == want.shape
        bad = np.nonzero(got != want)
        assert bad[0].size == 0, [(hex(int(got[i, j])), hex(int(want[i, j]))) for i, j in zip(*bad)][:5]


def tokens(seed: int, count: int) -> list[bytes]:
    rng = random.Random(seed)
    getcontext().prec = 200
    out = []
    for _ in range(count):
        r = rng.random()
        f = np.float32(np.frombuffer(rng.getrandbits(32).to_bytes(4, "little"), np.float32)[0])
        if not np.isfinite(f):
            f = np.float32(rng.uniform(-1e3, 1e3))
        if r < 0.25:   # the shortest forms and fixed precisions
            out.append(("%.*g" % (rng.randint(1, 12), float(f))).encode())
        elif r < 0.4:
            out.append(("%.*e" % (rng.randint(0, 30), float(f))).encode())
        elif r < 0.6:   # halfway between two adjacent floats, and next to it
            g = np.nextafter(f, np.float32(np.inf), dtype=np.float32)
            if not np.isfinite(g):
                g = np.nextafter(f, np.float32(-np.inf), dtype=np.float32)
            mid = (Decimal(float(f)) + Decimal(float(g))) / 2
            s = format(mid, "f") if abs(mid) > Decimal("1e-10") and abs(mid) < Decimal("1e20") else format(mid, "e")
            t = rng.random()
            if t < 0.4:
                out.append(s.encode())
            else:
                # a little above / below the midpoint in the last of many digits
                d = Decimal(10) ** (mid.adjusted() - rng.randint(25, 60))
                out.append(format(mid + (d if t < 0.7 else -d), "e").encode())
        elif r < 0.7:   # subnormal range and around the extremes
            e = rng.choice([-46, -45, -44, -40, -39, -38, 37, 38, 39])
            out.append(f"{rng.choice('+-')}{rng.randint(1, 99999)}.{rng.randint(0, 999999)}e{e}".encode())
        elif r < 0.8:   # long digit strings
            digits = "".join(rng.choice("0123456789") for _ in range(rng.randint(20, 60)))
            p = rng.randint(0, len(digits))
            out.append((digits[:p] + "." + digits[p:] + rng.choice(["", "e-7", "E+3", "e-30"])).encode())
        elif r < 0.9:   # integers, zeros, signs, leading zeros
            out.append(rng.choice([b"0", b"-0", b"+0.000", b"00012", b".5", b"5.", b"+.5e+2", b"-7e0", b"1e39",
                                   b"-1e-400", b"1e400", b"16777217", b"4294967297", b"0.1", b"1.000000059604644775390625"]))
        else:          # spellings for the host
            out.append(rng.choice([b"inf", b"-INF", b"Infinity", b"+infinity", b"nan", b"-nan", b"NaN(123)",
                                   b"0x1.8p3", b"-0x.1p-2", b"0X1P-149", b"0x1.fffffep127"]))
    return out


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_values_bit_for_bit(seed):
    toks = tokens(seed, 60000)
    rng = random.Random(seed)
    seps = [b" ", b",", b"\t", b";", b" , ", b"\v", b"\f", b"\r"]
    lines = []
    for i in range(0, len(toks) - len(toks) % 6, 6):
        lines.append(rng.choice(seps).join(toks[i:i + 6]) + rng.choice([b"", b" ", b"\r", b" # note"]))
    same(b"\n".join(lines) + b"\n")


def test_layout():
    """Comments, separators, CRLF, BOM, blank lines, '#' inside a token and
    across 32-byte chunks, long lines, no final newline."""
    long_line = b" ".join(b"%d.5" % i for i in range(5000))
    cases = [
        b"\xef\xbb\xbf1 2 3\n4,5,6\n",
        b"# header\n\n1;2;3 # tail\n  \t\n4\t5\t6\r\n7 8 9",
        b"1 2\n3 4#5 6\n",
        b"1.5#x 2\n3 4\n",
        b"1" * 40 + b".25 " + b"2" * 29 + b"#" + b"3" * 40 + b"\n1 2\n",
        b" " * 31 + b"1.5 2.5\n" + b" " * 30 + b"3 4\n",
        long_line + b"\n" + long_line + b"\n",
        b"",
        b"\n\n# only comments\n",
        b"1e-50 -1e-50 1e50\n",
    ]
    for raw in cases:
        same(raw)


def test_errors_in_file_order():
    cases = [
        b"1 2 3\n4 5\n6 x 7\n",          # inconsistent row first
        b"1 2 3\n4 x 6\n7 8\n",           # bad token first
        b"1 2 3\n4 5 bad 6\n",            # bad token on the inconsistent line: reported first
        b"1 2\n3 4\n5 6 7\n",
        b"1_000 2\n",
        b"1.5e 2\n",
        b"0x1p3 nan(abc) 1\n2 3 --1\n",
        b"1 2\n\n# c\n3 4 5 # x\n",
    ]
    for raw in cases:
        same(raw)
