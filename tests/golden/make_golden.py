"""Generate the committed golden fixtures from the reference itself.

Run in a checkout where the reference tree exists (``T1M_REFERENCE_DIR``,
default: a ``reference`` directory beside this repository's root):

    python tests/golden/make_golden.py

It writes

* ``unit_vectors.json`` — every known-answer vector of the reference's unit
  tests for the hot path (test/test_scatter.cpp, test/test_packing.cpp): the
  inputs each test builds and the expected arrays, parsed from the test
  sources, each cross-checked against the compiled reference (oracle/_ref).
* ``contractions.npz`` — seeded small contractions (the workload shapes at
  reduced extents, the reference's gemm-like test shapes, row-major cases)
  with the reference's output on them.

The fixtures are small; the GPU tests compare against them without the
reference tree.
"""
from __future__ import annotations

import json
import os
import re
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import libs  # noqa: E402
from oracle import numpy_oracle as no  # noqa: E402

REF = Path(os.environ.get("T1M_REFERENCE_DIR",
                          str(Path(__file__).resolve().parents[3] / "reference")))
OUT = Path(__file__).resolve().parent


# ----------------------------------------------------------- source parse ---
def _braced(text: str, start: int) -> str:
    """Text between the brace at ``start`` and its matching close brace."""
    depth = 0
    for i in range(start, len(text)):
        if text[i] == "{":
            depth += 1
        elif text[i] == "}":
            depth -= 1
            if depth == 0:
                return text[start + 1:i]
    raise ValueError("unbalanced braces")


def _numbers(s: str) -> list[float]:
    return [float(x) for x in re.findall(r"-?\d+(?:\.\d+)?", s)]


def _test_body(src: str, name: str) -> tuple[str, int]:
    m = re.search(r"TEST\(\w+,\s*%s\)\s*\{" % name, src)
    line = src[:m.start()].count("\n") + 1
    return _braced(src, m.end() - 1), line


def _expected_array(body: str) -> list[float]:
    m = re.search(r"expt\s*\{", body)
    return _numbers(_braced(body, m.end() - 1))


def _expect_vectors(body: str) -> dict[str, list[int]]:
    out = {}
    for m in re.finditer(r"EXPECT_EQ\((\w+(?:\.\w+)?),\s*\(std::vector<std::size_t>\{([^}]*)\}\)\)", body):
        out[m.group(1)] = [int(x) for x in _numbers(m.group(2))]
    return out


# ------------------------------------------------------------- unit cases ---
def unit_vectors() -> dict:
    scat_src = (REF / "test" / "test_scatter.cpp").read_text()
    pack_src = (REF / "test" / "test_packing.cpp").read_text()
    cases = []

    # Index bundles (test_scatter.cpp IndexBundling1/2).
    for name, labels in (("IndexBundling1", ("abc", "cd", "abd")),
                         ("IndexBundling2", ("abcde", "bdcf", "fae"))):
        body, line = _test_body(scat_src, name)
        exp = _expect_vectors(body)
        want = {k.replace(".", ""): v for k, v in exp.items()}
        got = libs.ref_index_bundles(*labels)
        assert all(got[k] == v for k, v in want.items()), (name, got, want)
        cases.append({"kind": "bundles", "name": name,
                      "source": f"test/test_scatter.cpp:{line}",
                      "labels": list(labels), "expected": want})

    # Scatter vectors on a 3x2x2x3 column-major tensor.
    body, line = _test_body(scat_src, "ScatterVectors")
    exp = _expect_vectors(body)
    dims = [3, 2, 2, 3]
    strides = no.col_major_strides(dims)
    for key, idx in (("rscat", [0, 1]), ("cscat", [2, 3])):
        got = libs.ref_scatter(idx, dims, strides).tolist()
        assert got == exp[key], (key, got, exp[key])
        cases.append({"kind": "scatter", "name": f"ScatterVectors.{key}",
                      "source": f"test/test_scatter.cpp:{line}", "dims": dims,
                      "indices": idx, "expected": exp[key]})

    # Block-scatter vectors.
    body, line = _test_body(scat_src, "BlockScatterVectors1")
    exp = _expect_vectors(body)
    for key, idx in (("block_rscat", [0, 1]), ("block_cscat", [2, 3])):
        sc = libs.ref_scatter(idx, dims, strides)
        got = libs.ref_block_scatter(sc, 3).tolist()
        assert got == exp[key], (key, got, exp[key])
        cases.append({"kind": "block_scatter", "name": f"BlockScatterVectors1.{key}",
                      "source": f"test/test_scatter.cpp:{line}",
                      "scatter": sc.tolist(), "b": 3, "expected": exp[key]})
    for name in ("BlockScatterVectors2", "BlockScatterVectors3", "BlockScatterVectors4"):
        body, line = _test_body(scat_src, name)
        m = re.search(r"scat\s*\{", body)
        sc = [int(x) for x in _numbers(_braced(body, m.end() - 1))]
        exp = _expect_vectors(body)["block_scat"]
        got = libs.ref_block_scatter(sc, 3).tolist()
        assert got == exp, (name, got, exp)
        cases.append({"kind": "block_scatter", "name": name,
                      "source": f"test/test_scatter.cpp:{line}", "scatter": sc,
                      "b": 3, "expected": exp})

    # Packing (real and 1M) and unpacking, test_packing.cpp.
    real_elems = np.arange(1, 17, dtype=np.float32)
    cplx_elems = np.array([complex(2 * i + 1, 2 * i + 2) for i in range(16)],
                          dtype=np.complex64)
    pack_cases = [
        # name, label, complex, dims, (X, Y), br, bc, length, dest_len
        ("PackColMajorEven", "A", False, [2, 2, 4], ([0, 1], [2]), 2, 2, 4, 16),
        ("PackColMajorOdd", "A", False, [2, 2, 4], ([0, 1], [2]), 3, 2, 4, 24),
        ("PackRowMajorEven", "B", False, [2, 2, 4], ([0, 1], [2]), 2, 2, 4, 16),
        ("PackRowMajorOdd", "B", False, [2, 2, 4], ([0, 1], [2]), 2, 3, 4, 24),
        ("Pack1MColMajorEven", "A", True, [2, 2, 4], ([0, 1], [2]), 4, 8, 8, 64),
        ("Pack1MColMajorOdd", "A", True, [2, 2, 4], ([0, 1], [2]), 6, 8, 8, 96),
        ("Pack1MRowMajorEven", "B", True, [2, 2, 4], ([0, 1], [2]), 8, 2, 8, 32),
        ("Pack1MRowMajorOdd", "B", True, [2, 2, 4], ([0, 1], [2]), 8, 3, 8, 48),
    ]
    for name, label, cpx, d, (bx, by), br, bc, length, dlen in pack_cases:
        body, line = _test_body(pack_src, name)
        exp = _expected_array(body)
        src = cplx_elems if cpx else real_elems
        got = libs.ref_pack_block(src, d, bx, by, br, bc, length, label, dlen)
        assert got.tolist() == exp, (name, got.tolist(), exp)
        cases.append({"kind": "pack", "name": name, "source": f"test/test_packing.cpp:{line}",
                      "label": label, "complex": cpx, "dims": d, "X": bx, "Y": by,
                      "br": br, "bc": bc, "length": length, "dest_len": dlen,
                      "expected": exp})
    # Unpack tests build a rank-3 tensor from two extents ({M, K}), so the
    # third extent is 0 and unused.
    for name, cpx, br, bc in (("Unpack", False, 4, 4), ("Unpack1M", True, 8, 8)):
        body, line = _test_body(pack_src, name)
        exp = _expected_array(body)
        d = [4, 4, 0]
        if cpx:
            src = cplx_elems.view(np.float32)
            dest = np.zeros(16, dtype=np.complex64)
            got = libs.ref_unpack(src, d, [1], [0], br, bc, dest)
            flat = np.stack([got.real, got.imag], axis=1).reshape(-1).tolist()
        else:
            src = real_elems
            dest = np.zeros(16, dtype=np.float32)
            flat = libs.ref_unpack(src, d, [1], [0], br, bc, dest).tolist()
        assert flat == exp, (name, flat, exp)
        cases.append({"kind": "unpack", "name": name, "source": f"test/test_packing.cpp:{line}",
                      "complex": cpx, "dims": d, "X": [1], "Y": [0], "br": br, "bc": bc,
                      "expected": exp})
    return {"generator": "tests/golden/make_golden.py", "cases": cases}


# ------------------------------------------------------- contraction cases ---
# (name, labels a/b/c, extents per label, dtypes, c_init)
CONTRACTIONS = [
    ("cfg1_abc_bd_acd", ("abc", "bd", "acd"), dict(a=10, b=10, c=10, d=10),
     ["c64"], "zero"),
    ("cfg2a_small", ("abcd", "efcd", "abef"), dict(a=6, b=5, c=4, d=7, e=3, f=6),
     ["c64", "c128"], "uniform"),
    ("cfg2b_small", ("abcd", "dbea", "ec"), dict(a=3, b=4, c=12, d=6, e=8),
     ["c64", "c128"], "uniform"),
    ("cfg3_small", ("ijkl", "klmn", "ijmn"), dict(i=5, j=6, k=7, l=4, m=3, n=5),
     ["c64"], "zero"),
    ("cfg4_step1_small", ("xay", "asb", "xsyb"), dict(x=5, a=6, y=4, s=2, b=7),
     ["c64"], "zero"),
    ("cfg4_step2_small", ("xsyb", "ytb", "xst"), dict(x=5, s=2, y=4, b=7, t=4),
     ["c64"], "zero"),
    ("cfg5_small", ("abcd", "ebfd", "aecf"), dict(a=4, b=3, c=5, d=4, e=3, f=4),
     ["c64"], "uniform"),
    ("gemm_ab_bc_ac", ("ab", "bc", "ac"), dict(a=5, b=5, c=5),
     ["f32", "f64", "c64", "c128"], "zero"),
    ("gemm_abc_bce_ae", ("abc", "bce", "ae"), dict(a=5, b=5, c=5, e=5),
     ["f32", "f64", "c64", "c128"], "zero"),
    ("gemm_abc_cd_abd", ("abc", "cd", "abd"), dict(a=5, b=5, c=5, d=5),
     ["f32", "f64", "c64", "c128"], "zero"),
    ("gemm_abc_cde_abde", ("abc", "cde", "abde"), dict(a=5, b=5, c=5, d=5, e=5),
     ["f32", "f64", "c64", "c128"], "zero"),
    ("gemm_abcd_cde_abe", ("abcd", "cde", "abe"), dict(a=5, b=5, c=5, d=5, e=5),
     ["f32", "f64", "c64", "c128"], "zero"),
    ("gemm_abcd_cdef_abef", ("abcd", "cdef", "abef"), dict(a=5, b=5, c=5, d=5, e=5, f=5),
     ["f32", "f64", "c64", "c128"], "zero"),
    ("permuted_bench_dbea_ec", ("dbea", "ec", "abcd"), dict(a=9, b=8, c=5, d=7, e=6),
     ["c64", "f32"], "uniform"),
    ("ragged_odd", ("zqa", "aqw", "wz"), dict(z=13, q=7, a=11, w=17),
     ["c64", "c128", "f32", "f64"], "uniform"),
]

DT = {"f32": np.float32, "f64": np.float64, "c64": np.complex64, "c128": np.complex128}


def _rand(rng, shape, dt):
    x = rng.uniform(-1.0, 1.0, size=shape)
    if np.dtype(dt).kind == "c":
        x = x + 1j * rng.uniform(-1.0, 1.0, size=shape)
    return x.astype(dt)


def contractions() -> dict:
    out = {}
    rng = np.random.default_rng(20240601)
    for name, (la, lb, lc), ext, dts, cinit in CONTRACTIONS:
        da = [ext[ch] for ch in la]
        db = [ext[ch] for ch in lb]
        dc = [ext[ch] for ch in lc]
        for dts_ in dts:
            dt = DT[dts_]
            for layout in ("col", "row"):
                A = _rand(rng, da, dt)
                B = _rand(rng, db, dt)
                C0 = _rand(rng, dc, dt) if cinit == "uniform" else np.zeros(dc, dt)
                alpha = 0.75 if dts_ in ("f32", "f64") else 1.0
                # Column-major buffers of the logical tensors; the row-major
                # case is the same bytes seen with reversed extents and labels.
                if layout == "col":
                    fa = A.reshape(-1, order="F").copy()
                    fb = B.reshape(-1, order="F").copy()
                    fc = C0.reshape(-1, order="F").copy()
                    libs.ref_contract(fa, da, la, fb, db, lb, fc, dc, lc, alpha, 0.0)
                    out_flat = fc
                    in_a = fa
                    in_b = fb
                    in_c = C0.reshape(-1, order="F").copy()
                else:
                    fa = A.reshape(-1, order="C").copy()
                    fb = B.reshape(-1, order="C").copy()
                    fc = C0.reshape(-1, order="C").copy()
                    libs.ref_contract(fa, da[::-1], la[::-1], fb, db[::-1], lb[::-1],
                                      fc, dc[::-1], lc[::-1], alpha, 0.0)
                    out_flat = fc
                    in_a = fa
                    in_b = fb
                    in_c = C0.reshape(-1, order="C").copy()
                key = f"{name}__{dts_}__{layout}"
                out[key + "__a"] = in_a
                out[key + "__b"] = in_b
                out[key + "__c0"] = in_c
                out[key + "__c"] = out_flat
                out[key + "__meta"] = np.array(json.dumps({
                    "labels": [la, lb, lc], "dims": [da, db, dc], "layout": layout,
                    "dtype": dts_, "alpha": alpha, "semantics": "C0 + alpha*A*B"}))
    return out


def main() -> None:
    uv = unit_vectors()
    (OUT / "unit_vectors.json").write_text(json.dumps(uv, indent=1) + "\n")
    np.savez_compressed(OUT / "contractions.npz", **contractions())
    print("wrote", OUT / "unit_vectors.json", OUT / "contractions.npz")


if __name__ == "__main__":
    main()
