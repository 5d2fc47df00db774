"""CPU checks of the boundary: the C-ABI library builds for sm_103a, loads, and
exports every function include/turbotops_gb300.h declares (no device calls)."""
import ctypes
import os
import re

from turbotops_gb300 import build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "turbotops_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tt_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    names = declared()
    assert len(names) >= 8
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(capi.exported_symbols())


def test_metric_parse_matches_reference_messages():
    assert capi.metric_parse("l2") == (1, 2.0)
    assert capi.metric_parse("manhattan") == (0, 1.0)
    assert capi.metric_parse("lp:1") == (0, 1.0)
    assert capi.metric_parse("lp:inf")[0] == 2
    k, p = capi.metric_parse("lp:1.5")
    assert k == 3 and abs(p - 1.5) < 1e-7
    import pytest
    with pytest.raises(ValueError, match="p must be in"):
        capi.metric_parse("lp:0.5")
    with pytest.raises(ValueError, match="unknown 'cosine'"):
        capi.metric_parse("cosine")
