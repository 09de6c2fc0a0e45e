"""CPU tests of the product library: it loads, exports every symbol that
include/*.h declares, and validates labels on the host (no GPU calls)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(?:int|const char\*)\s+(t1m_\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    syms = _declared_symbols()
    for s in ("t1m_create", "t1m_destroy", "t1m_contract", "t1m_analyze", "t1m_set_stream",
              "t1m_set_method", "t1m_status_string", "t1m_last_error", "t1m_version"):
        assert s in syms


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(str(built_lib))
    missing = [s for s in _declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_library_is_sm103a_only(built_lib):
    import t1m_gb300 as t1m
    assert t1m.version()[2] == 103
    from t1m_gb300 import build as b
    assert "arch=compute_103a,code=sm_103a" in b.ARCH


def test_no_device_is_an_error_not_a_fallback(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import t1m_gb300 as t1m
    with pytest.raises(t1m.T1MError) as e:
        t1m.Context()
    assert e.value.status == 7


def _t(dims, dt=np.complex64):
    import t1m_gb300 as t1m
    return t1m.tensor(list(dims), np.zeros(max(1, int(np.prod(dims))), dt))


@pytest.mark.parametrize("la,lb,lc,da,db,dc,mnk", [
    ("abc", "bd", "acd", (10, 10, 10), (10, 10), (10, 10, 10), (100, 10, 10)),
    ("abcd", "efcd", "abef", (48,) * 4, (48,) * 4, (48,) * 4, (2304, 2304, 2304)),
    ("abcd", "dbea", "ec", (24, 32, 96, 48), (48, 32, 64, 24), (64, 96), (96, 64, 36864)),
    ("ijkl", "klmn", "ijmn", (64,) * 4, (64,) * 4, (64,) * 4, (4096, 4096, 4096)),
    ("ab", "cd", "abcd", (3, 4), (5, 6), (3, 4, 5, 6), (12, 30, 1)),   # outer product
    ("ab", "ab", "", (3, 4), (3, 4), (), (1, 1, 12)),                   # full contraction
    ("abc", "bc", "ac", (2, 3, 4), (3, 4), (2, 4), (2, 1, 3)),          # batch label c
])
def test_analyze_sizes(built_lib, la, lb, lc, da, db, dc, mnk):
    import t1m_gb300 as t1m
    info = t1m.analyze(_t(da), la, _t(db), lb, _t(dc), lc)
    assert (info["m"], info["n"], info["k"]) == mnk


@pytest.mark.parametrize("la,lb,lc,da,db,dc,msg", [
    ("abb", "bd", "ad", (2, 3, 3), (3, 4), (2, 4), "repeated"),
    ("abc", "bd", "acd", (2, 3, 4), (5, 4), (2, 4, 4), "extent mismatch"),
    ("abc", "cd", "ad", (2, 3, 4), (4, 5), (2, 5), "missing from C"),
    ("abc", "bc", "ac", (2, 3, 4), (3, 5), (2, 4), "batch label"),
    ("ab", "bc", "acz", (2, 3), (3, 4), (2, 4, 5), "neither A nor B"),
    ("ab", "bc", "a", (2, 3), (3, 4), (2,), "missing from C"),
    ("a#", "bc", "ac", (2, 3), (3, 4), (2, 4), "invalid label"),
    ("ab", "bc", "ac", (2, 3, 4), (3, 4), (2, 4), "length differs"),
])
def test_analyze_rejects_bad_labels(built_lib, la, lb, lc, da, db, dc, msg):
    import t1m_gb300 as t1m
    with pytest.raises(t1m.T1MError) as e:
        t1m.analyze(_t(da), la, _t(db), lb, _t(dc), lc)
    assert msg in str(e.value)


def test_analyze_matches_numpy_restatement_bundle_sizes(built_lib):
    import t1m_gb300 as t1m
    from oracle import numpy_oracle as no
    rng = np.random.default_rng(5)
    for _ in range(20):
        letters = list("abcdefg")
        rng.shuffle(letters)
        la, lb = "".join(letters[:4]), "".join(letters[2:6])
        lc = "".join(sorted(set(la) ^ set(lb)))
        ext = {ch: int(rng.integers(1, 5)) for ch in letters}
        da, db, dc = ([ext[ch] for ch in s] for s in (la, lb, lc))
        bd = no.index_bundles(la, lb, lc)
        m = int(np.prod([da[i] for i in bd["AX"]]))
        n = int(np.prod([db[i] for i in bd["BY"]]))
        k = int(np.prod([da[i] for i in bd["AY"]]))
        info = t1m.analyze(_t(da), la, _t(db), lb, _t(dc), lc)
        assert (info["m"], info["n"], info["k"]) == (m, n, k)
