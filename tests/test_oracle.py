"""CPU tests of the oracle itself (no GPU).

Pins the numpy restatement and the C++ port against
  * every known-answer vector of the reference's unit tests
    (tests/golden/unit_vectors.json, from test/test_scatter.cpp and
    test/test_packing.cpp),
  * the reference's own outputs on seeded contractions
    (tests/golden/contractions.npz),
  * the unmodified reference itself (oracle/_ref), where it was built here.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import libs
from oracle import numpy_oracle as no

GOLDEN = Path(__file__).resolve().parent / "golden"
UNIT = json.loads((GOLDEN / "unit_vectors.json").read_text())["cases"]
FIX = np.load(GOLDEN / "contractions.npz")
FIX_KEYS = sorted({k.rsplit("__", 1)[0] for k in FIX.files})


def _case_id(c):
    return c["name"]


@pytest.mark.parametrize("case", UNIT, ids=_case_id)
def test_unit_vector_numpy_restatement(case):
    kind = case["kind"]
    if kind == "bundles":
        got = no.index_bundles(*case["labels"])
        for k, v in case["expected"].items():
            assert got[k] == v
    elif kind == "scatter":
        d = case["dims"]
        got = no.scatter(case["indices"], d, no.col_major_strides(d))
        assert got.tolist() == case["expected"]
    elif kind == "block_scatter":
        assert no.block_scatter(case["scatter"], case["b"]).tolist() == case["expected"]
    elif kind == "pack":
        n = int(np.prod(case["dims"]))
        if case["complex"]:
            src = np.array([complex(2 * i + 1, 2 * i + 2) for i in range(n)], np.complex64)
        else:
            src = np.arange(1, n + 1, dtype=np.float32)
        got = no.pack_block(src, case["dims"], case["X"], case["Y"], case["br"], case["bc"],
                            case["length"], case["label"], case["complex"], case["dest_len"])
        assert got.tolist() == case["expected"]
    elif kind == "unpack":
        if case["complex"]:
            src = np.array([complex(2 * i + 1, 2 * i + 2) for i in range(16)],
                           np.complex64).view(np.float32)
            got = no.unpack(src, case["dims"], case["X"], case["Y"], case["br"],
                            np.zeros(16, np.complex64), True)
            flat = np.stack([got.real, got.imag], 1).reshape(-1).tolist()
        else:
            src = np.arange(1, 17, dtype=np.float32)
            flat = no.unpack(src, case["dims"], case["X"], case["Y"], case["br"],
                             np.zeros(16, np.float32), False).tolist()
        assert flat == case["expected"]
    else:
        pytest.fail(kind)


def test_unit_vectors_cover_reference_tests():
    names = {c["name"].split(".")[0] for c in UNIT}
    assert {"IndexBundling1", "IndexBundling2", "ScatterVectors", "BlockScatterVectors1",
            "BlockScatterVectors2", "BlockScatterVectors3", "BlockScatterVectors4",
            "PackColMajorEven", "PackColMajorOdd", "PackRowMajorEven", "PackRowMajorOdd",
            "Unpack", "Pack1MColMajorEven", "Pack1MColMajorOdd", "Pack1MRowMajorEven",
            "Pack1MRowMajorOdd", "Unpack1M"} <= names


def _fixture(key):
    meta = json.loads(str(FIX[key + "__meta"]))
    return meta, FIX[key + "__a"], FIX[key + "__b"], FIX[key + "__c0"], FIX[key + "__c"]


def _strides(dims, layout):
    return no.col_major_strides(dims) if layout == "col" else no.row_major_strides(dims)


@pytest.mark.parametrize("key", FIX_KEYS)
def test_port_matches_reference_fixture_bitwise(key):
    """The C++ port reproduces the reference's bits on its golden outputs."""
    meta, fa, fb, fc0, fc = _fixture(key)
    (la, lb, lc), (da, db, dc) = meta["labels"], meta["dims"]
    L = meta["layout"]
    c = fc0.copy()
    libs.port_contract(fa, da, _strides(da, L), la, fb, db, _strides(db, L), lb, c, dc,
                       _strides(dc, L), lc, alpha=meta["alpha"], beta=0.0)
    assert np.array_equal(c.view(np.uint8), fc.view(np.uint8))


@pytest.mark.parametrize("key", FIX_KEYS)
def test_reference_fixture_against_fp64(key):
    """The golden outputs are within FP rounding of the FP64 oracle."""
    meta, fa, fb, fc0, fc = _fixture(key)
    (la, lb, lc), (da, db, dc) = meta["labels"], meta["dims"]
    order = "F" if meta["layout"] == "col" else "C"
    A = fa.reshape(da, order=order)
    B = fb.reshape(db, order=order)
    C0 = fc0.reshape(dc, order=order)
    ref = no.contract_fp64(A, la, B, lb, C0, lc, alpha=meta["alpha"], accumulate=True)
    mx, fro = no.rel_errors(fc.reshape(dc, order=order), ref)
    tol = 1e-5 if fa.dtype in (np.float32, np.complex64) else 1e-13
    assert mx < tol and fro < tol


def test_port_threads_do_not_change_bits():
    rng = np.random.default_rng(3)
    da, db, dc = (40, 30, 20), (20, 50), (40, 30, 50)
    fa = (rng.uniform(-1, 1, 24000) + 1j * rng.uniform(-1, 1, 24000)).astype(np.complex64)
    fb = (rng.uniform(-1, 1, 1000) + 1j * rng.uniform(-1, 1, 1000)).astype(np.complex64)
    outs = []
    for nt in (1, 3, 4):
        c = np.zeros(60000, np.complex64)
        libs.port_contract(fa, da, no.col_major_strides(da), "abc", fb, db,
                           no.col_major_strides(db), "cd", c, dc, no.col_major_strides(dc),
                           "abd", nthreads=nt)
        outs.append(c)
    assert all(np.array_equal(outs[0], o) for o in outs[1:])


ref_only = pytest.mark.skipif(libs.ref_lib() is None,
                              reason="reference tree absent (shim only builds where it exists)")


@ref_only
@pytest.mark.parametrize("seed", range(6))
def test_numpy_restatement_matches_reference_internals(seed):
    """Random bundles / scatter / block-scatter against the reference's own
    functions (t1m.h:90-205)."""
    rng = np.random.default_rng(seed)
    letters = list("abcdefgh")
    rng.shuffle(letters)
    la = "".join(letters[:4])
    lb = "".join(letters[2:6])
    lc = "".join(sorted(set(la) ^ set(lb), key=lambda ch: rng.random()))
    assert libs.ref_index_bundles(la, lb, lc) == no.index_bundles(la, lb, lc)
    dims = [int(x) for x in rng.integers(1, 6, size=4)]
    strides = no.col_major_strides(dims)
    for idx in ([0, 1], [2, 3], [3, 1, 0], [2]):
        s_ref = libs.ref_scatter(idx, dims, strides)
        assert s_ref.tolist() == no.scatter(idx, dims, strides).tolist()
        for b in (2, 3, 4):
            assert libs.ref_block_scatter(s_ref, b).tolist() == no.block_scatter(s_ref, b).tolist()


@ref_only
@pytest.mark.parametrize("dt", [np.float32, np.float64, np.complex64, np.complex128])
def test_port_matches_reference_on_benchmark_shape(dt):
    """A permuted shape from the reference's benchmark suite, port vs reference bits."""
    rng = np.random.default_rng(7)
    la, lb, lc = "dbea", "ec", "abcd"
    ext = dict(a=9, b=8, c=6, d=7, e=10)
    da, db, dc = [[ext[ch] for ch in s] for s in (la, lb, lc)]

    def r(n):
        x = rng.uniform(-1, 1, n)
        if np.dtype(dt).kind == "c":
            x = x + 1j * rng.uniform(-1, 1, n)
        return x.astype(dt)

    fa, fb, fc = r(int(np.prod(da))), r(int(np.prod(db))), r(int(np.prod(dc)))
    c1, c2 = fc.copy(), fc.copy()
    libs.port_contract(fa, da, no.col_major_strides(da), la, fb, db, no.col_major_strides(db),
                       lb, c1, dc, no.col_major_strides(dc), lc, alpha=0.5, beta=0.0)
    libs.ref_contract(fa, da, la, fb, db, lb, c2, dc, lc, alpha=0.5, beta=0.0)
    assert np.array_equal(c1.view(np.uint8), c2.view(np.uint8))
