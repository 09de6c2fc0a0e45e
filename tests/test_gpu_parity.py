"""GPU parity of the contraction engine against the oracle (marked gpu).

Every case goes through the C-ABI (libt1m_cuda.so via t1m_gb300) and is
compared with
  * the reference's own outputs on the committed seeded inputs
    (tests/golden/contractions.npz, generated by the unmodified reference), and
  * the FP64 oracle (full einsum at small sizes, sampled FP64 dot products at
    the full workload sizes).

Tolerances (normwise max relative error, max|dC| / max|C|):
  FP32 paths (plain, 3xTF32): 2e-5 at fixture sizes (K <= 500), the measured
  budget per method at the full sizes; FP64 paths: 1e-12.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import numpy_oracle as no

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
FIX = np.load(GOLDEN / "contractions.npz")
FIX_KEYS = sorted({k.rsplit("__", 1)[0] for k in FIX.files})

TOL = {np.dtype(np.float32): 2e-5, np.dtype(np.complex64): 2e-5,
       np.dtype(np.float64): 1e-12, np.dtype(np.complex128): 1e-12}


def _layout(t1m, L):
    return t1m.col_major if L == "col" else t1m.row_major


def _fixture(key):
    meta = json.loads(str(FIX[key + "__meta"]))
    return meta, FIX[key + "__a"], FIX[key + "__b"], FIX[key + "__c0"], FIX[key + "__c"]


def _methods_for(dtype):
    ms = ["plain"]
    if np.dtype(dtype) == np.complex64:
        ms.append("tc_3xtf32")
    if np.dtype(dtype) in (np.complex128, np.float64):
        ms.append("dmma")
    return ms


@pytest.mark.parametrize("key", FIX_KEYS)
def test_reference_semantics_host_buffers(ctx, key):
    """t1m.contract on host buffers == the reference's output (C += A*B)."""
    import t1m_gb300 as t1m
    meta, fa, fb, fc0, fc = _fixture(key)
    (la, lb, lc), (da, db, dc) = meta["labels"], meta["dims"]
    L = _layout(t1m, meta["layout"])
    for m in _methods_for(fa.dtype):
        ctx.set_method("plain" if m == "plain" else m)
        c = fc0.copy()
        a, b, cc = t1m.tensor(da, fa, L), t1m.tensor(db, fb, L), t1m.tensor(dc, c, L)
        try:
            if fa.dtype.kind == "c":
                rep = t1m.contract(a, la, b, lb, cc, lc, ctx=ctx)
            else:
                rep = t1m.contract(meta["alpha"], a, la, b, lb, 0.0, cc, lc, ctx=ctx)
        except t1m.T1MError as e:
            if e.status == 5 and m != "plain":
                continue  # method not available for this shape
            raise
        scale = max(np.abs(fc).max(), 1e-30)
        err = np.abs(c.astype(np.complex128) - fc.astype(np.complex128)).max() / scale
        assert err < TOL[fa.dtype], (m, err)
        assert rep.kernels >= 1
    ctx.set_method("auto")


@pytest.mark.parametrize("key", [k for k in FIX_KEYS if "__c64__" in k or "__c128__" in k])
def test_device_buffers_blas_semantics(ctx, torch_cuda, key):
    """Device (torch) buffers, C = alpha*A*B + beta*C with complex alpha/beta."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    meta, fa, fb, fc0, _ = _fixture(key)
    (la, lb, lc), (da, db, dc) = meta["labels"], meta["dims"]
    L = _layout(t1m, meta["layout"])
    order = "F" if meta["layout"] == "col" else "C"
    alpha, beta = 1 + 0.5j, 0.25
    ref = no.contract_fp64(fa.reshape(da, order=order), la, fb.reshape(db, order=order), lb,
                           fc0.reshape(dc, order=order), lc, alpha=alpha, beta=beta)
    for m in _methods_for(fa.dtype):
        ctx.set_method(m)
        ga = torch.from_numpy(fa).cuda()
        gb = torch.from_numpy(fb).cuda()
        gc = torch.from_numpy(fc0.copy()).cuda()
        try:
            t1m.contract_scaled(alpha, t1m.tensor(da, ga, L), la, t1m.tensor(db, gb, L), lb,
                                beta, t1m.tensor(dc, gc, L), lc, ctx=ctx)
        except t1m.T1MError as e:
            if e.status == 5 and m != "plain":
                continue
            raise
        torch.cuda.synchronize()
        got = gc.cpu().numpy().reshape(dc, order=order)
        mx, fro = no.rel_errors(got, ref)
        assert mx < TOL[fa.dtype] and fro < TOL[fa.dtype], (m, mx, fro)
    ctx.set_method("auto")


def _rand(rng, n, dt):
    x = rng.uniform(-1, 1, n)
    if np.dtype(dt).kind == "c":
        x = x + 1j * rng.uniform(-1, 1, n)
    return x.astype(dt)


def _sampled_check(fa, fb, fc_out, fc0, la, lb, lc, da, db, dc, strides, alpha, beta,
                   samples=1024, seed=0):
    """Normwise errors at sampled C entries against FP64 dot products."""
    sa, sb, sc = strides
    scat = no.matricize(la, lb, lc, da, db, dc, sa, sb, sc)
    M, N = len(scat[0]), len(scat[3])
    rng = np.random.default_rng(seed)
    rows = rng.integers(0, M, samples)
    cols = rng.integers(0, N, samples)
    ab = no.sampled_entries(fa, fb, scat, rows, cols)
    offc = scat[4][rows] + scat[5][cols]
    ref = alpha * ab + beta * fc0[offc].astype(np.complex128)
    got = fc_out[offc].astype(np.complex128)
    return no.rel_errors(got, ref)


def plain_tol(k, split_k=1):
    """Error budget of the plain FP32 form: 4 u sqrt(2K/split) (u = 2^-24),
    at least 2e-5."""
    return max(2e-5, 4 * 2.0 ** -24 * np.sqrt(2.0 * k / max(1, split_k)))


CFG2 = [
    ("abcd", "efcd", "abef", dict(a=48, b=48, c=48, d=48, e=48, f=48)),
    ("abcd", "dbea", "ec", dict(a=24, b=32, c=96, d=48, e=64)),
]


@pytest.mark.slow
@pytest.mark.parametrize("dt", [np.complex64, np.complex128])
@pytest.mark.parametrize("layout", ["col", "row"])
@pytest.mark.parametrize("cfg", range(len(CFG2)))
def test_config2_full_size_plain(ctx, torch_cuda, cfg, layout, dt):
    """The plain drop-in workload at full size: abcd,efcd->abef (48^4) and the
    permuted abcd,dbea->ec, col- and row-major, alpha = 1+0.5i, beta = 0.25."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    la, lb, lc, ext = CFG2[cfg]
    da, db, dc = ([ext[ch] for ch in s] for s in (la, lb, lc))
    strides = [(no.col_major_strides if layout == "col" else no.row_major_strides)(d)
               for d in (da, db, dc)]
    rng = np.random.default_rng(11)
    fa, fb = _rand(rng, int(np.prod(da)), dt), _rand(rng, int(np.prod(db)), dt)
    fc0 = _rand(rng, int(np.prod(dc)), dt)
    alpha, beta = 1 + 0.5j, 0.25
    ctx.set_method("plain")
    L = _layout(t1m, layout)
    ga, gb, gc = (torch.from_numpy(x.copy()).cuda() for x in (fa, fb, fc0))
    rep = t1m.contract_scaled(alpha, t1m.tensor(da, ga, L), la, t1m.tensor(db, gb, L), lb,
                              beta, t1m.tensor(dc, gc, L), lc, ctx=ctx)
    torch.cuda.synchronize()
    out = gc.cpu().numpy()
    mx, fro = _sampled_check(fa, fb, out, fc0, la, lb, lc, da, db, dc, strides, alpha, beta)
    # Plain FP32 accumulates K sequentially in one register per output, so its
    # error grows like u*sqrt(2K) (u = 2^-24); split-K with an FP64 reduction
    # is what brings long contractions under 1e-6.
    tol = plain_tol(rep.k, rep.split_k) if dt == np.complex64 else 1e-12
    assert mx < tol and fro < tol, (mx, fro, tol)
    assert rep.method == 1
    ctx.set_method("auto")


@pytest.mark.slow
@pytest.mark.parametrize("layout", ["col", "row"])
@pytest.mark.parametrize("cfg", range(len(CFG2)))
def test_config2_full_size_tensor_core(ctx, torch_cuda, cfg, layout):
    """complex64 config 2 on the tensor cores (3xTF32, automatic split-K for the
    skinny permuted case): the 1e-6 bar against sampled FP64."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    la, lb, lc, ext = CFG2[cfg]
    da, db, dc = ([ext[ch] for ch in s] for s in (la, lb, lc))
    strides = [(no.col_major_strides if layout == "col" else no.row_major_strides)(d)
               for d in (da, db, dc)]
    rng = np.random.default_rng(12)
    dt = np.complex64
    fa, fb = _rand(rng, int(np.prod(da)), dt), _rand(rng, int(np.prod(db)), dt)
    fc0 = _rand(rng, int(np.prod(dc)), dt)
    alpha, beta = 1 + 0.5j, 0.25
    ctx.set_method("tc_3xtf32")
    L = _layout(t1m, layout)
    ga, gb, gc = (torch.from_numpy(x.copy()).cuda() for x in (fa, fb, fc0))
    rep = t1m.contract_scaled(alpha, t1m.tensor(da, ga, L), la, t1m.tensor(db, gb, L), lb,
                              beta, t1m.tensor(dc, gc, L), lc, ctx=ctx)
    torch.cuda.synchronize()
    mx, fro = _sampled_check(fa, fb, gc.cpu().numpy(), fc0, la, lb, lc, da, db, dc, strides,
                             alpha, beta)
    assert mx < 1e-6 and fro < 1e-6, (mx, fro, rep.split_k)
    assert rep.method == 2
    if cfg == 1:
        # Split-K with its FP64 reduction, after dense packs of the operands
        # that would be gathered element by element: A (col-major), A and B
        # (row-major, where B's 24-element runs of a straddle 16-element blocks).
        assert rep.split_k > 1 and rep.kernels == (3 if layout == "col" else 4), rep.kernels
    ctx.set_method("auto")


@pytest.mark.parametrize("method", ["plain", "tc_3xtf32"])
@pytest.mark.parametrize("splits", [2, 3, 7])
@pytest.mark.parametrize("key", ["cfg2b_small__c64__col", "cfg3_small__c64__row",
                                 "ragged_odd__c64__col", "ragged_odd__f64__row",
                                 "cfg2a_small__c128__col"])
def test_forced_split_k(ctx, key, splits, method):
    """Split-K (partials in a workspace, FP64 reduction) gives the same result
    as the reference on the committed fixtures, for any split count."""
    import t1m_gb300 as t1m
    meta, fa, fb, fc0, fc = _fixture(key)
    if method != "plain" and fa.dtype != np.complex64:
        pytest.skip("tensor-core method is complex64")
    (la, lb, lc), (da, db, dc) = meta["labels"], meta["dims"]
    L = _layout(t1m, meta["layout"])
    ctx.set_method(method)
    ctx.set_split_k(splits)
    try:
        c = fc0.copy()
        a, b, cc = t1m.tensor(da, fa, L), t1m.tensor(db, fb, L), t1m.tensor(dc, c, L)
        if fa.dtype.kind == "c":
            rep = t1m.contract(a, la, b, lb, cc, lc, ctx=ctx)
        else:
            rep = t1m.contract(meta["alpha"], a, la, b, lb, 0.0, cc, lc, ctx=ctx)
    finally:
        ctx.set_split_k(0)
        ctx.set_method("auto")
    assert rep.split_k > 1 or rep.k <= 16
    scale = max(np.abs(fc).max(), 1e-30)
    err = np.abs(c.astype(np.complex128) - fc.astype(np.complex128)).max() / scale
    assert err < TOL[fa.dtype], err


def test_edge_cases(ctx, torch_cuda):
    """Zero extents, an outer product (empty K), a full contraction to a
    0-mode C, and non-contiguous views."""
    import t1m_gb300 as t1m
    rng = np.random.default_rng(2)
    ctx.set_method("plain")
    # Outer product ab,cd->acbd.
    A = _rand(rng, 12, np.complex64).reshape(3, 4)
    B = _rand(rng, 30, np.complex64).reshape(5, 6)
    C = np.zeros((3, 5, 4, 6), np.complex64)
    t1m.contract_scaled(1.0, t1m.tensor.from_array(A), "ab", t1m.tensor.from_array(B), "cd",
                        0.0, t1m.tensor.from_array(C), "acbd", ctx=ctx)
    np.testing.assert_allclose(C, np.einsum("ab,cd->acbd", A, B), rtol=1e-6, atol=1e-6)
    # Full contraction to a scalar.
    A = _rand(rng, 60, np.complex128).reshape(3, 4, 5)
    B = _rand(rng, 60, np.complex128).reshape(3, 4, 5)
    c = np.zeros((), np.complex128)
    t1m.contract_scaled(1.0, t1m.tensor.from_array(A), "abc", t1m.tensor.from_array(B),
                        "abc", 0.0, t1m.tensor.from_array(c), "", ctx=ctx)
    assert abs(c - np.einsum("abc,abc->", A, B)) < 1e-12
    # Zero extent: C untouched under accumulate, zeroed under beta = 0.
    A = np.zeros((0, 4), np.float32)
    B = _rand(rng, 20, np.float32).reshape(4, 5)
    C = np.ones((0, 5), np.float32)
    t1m.contract_scaled(1.0, t1m.tensor.from_array(A), "ab", t1m.tensor.from_array(B), "bc",
                        0.0, t1m.tensor.from_array(C), "ac", ctx=ctx)
    A = np.zeros((3, 0), np.float32)
    B = np.zeros((0, 5), np.float32)
    C = np.ones((3, 5), np.float32)
    t1m.contract(1.0, t1m.tensor.from_array(A), "ab", t1m.tensor.from_array(B), "bc", 0.0,
                 t1m.tensor.from_array(C), "ac", ctx=ctx)
    assert np.all(C == 1.0)
    t1m.contract_scaled(1.0, t1m.tensor.from_array(A), "ab", t1m.tensor.from_array(B), "bc",
                        0.0, t1m.tensor.from_array(C), "ac", ctx=ctx)
    assert np.all(C == 0.0)
    # Non-contiguous views (every other element, transposed).
    big = _rand(rng, 2 * 7 * 9, np.complex64).reshape(7, 18)
    A = big[:, ::2]                     # (7, 9) with strides (18, 2)
    B = _rand(rng, 9 * 11, np.complex64).reshape(11, 9).T   # (9, 11) transposed
    Cbig = np.zeros((7, 22), np.complex64)
    Cv = Cbig[:, 1::2]
    t1m.contract_scaled(2.0, t1m.tensor.from_array(A), "ik", t1m.tensor.from_array(B), "kj",
                        0.0, t1m.tensor.from_array(Cv), "ij", ctx=ctx)
    np.testing.assert_allclose(Cv, 2.0 * A @ B, rtol=2e-6, atol=2e-6)
    assert np.all(Cbig[:, 0::2] == 0)
    ctx.set_method("auto")


@pytest.mark.parametrize("conj", [(False, True), (True, False), (True, True)])
def test_conjugation_flags(ctx, conj):
    import t1m_gb300 as t1m
    rng = np.random.default_rng(4)
    A = _rand(rng, 6 * 7 * 5, np.complex64).reshape(6, 7, 5)
    B = _rand(rng, 5 * 7 * 8, np.complex64).reshape(5, 7, 8)
    C = np.zeros((6, 8), np.complex64)
    t1m.contract_scaled(1.0, t1m.tensor.from_array(A), "abc", t1m.tensor.from_array(B), "cbd",
                        0.0, t1m.tensor.from_array(C), "ad", ctx=ctx, conj_a=conj[0],
                        conj_b=conj[1])
    Ar = np.conj(A) if conj[0] else A
    Br = np.conj(B) if conj[1] else B
    np.testing.assert_allclose(C, np.einsum("abc,cbd->ad", Ar, Br), rtol=1e-5, atol=1e-5)


def test_errors_are_reported_not_crashing(ctx):
    import t1m_gb300 as t1m
    A = np.zeros((2, 3), np.complex64)
    with pytest.raises(t1m.T1MError) as e:
        # label d of C appears in neither A nor B
        t1m.contract_scaled(1.0, t1m.tensor.from_array(A), "ab", t1m.tensor.from_array(A.T.copy()),
                            "bc", 0.0, t1m.tensor.from_array(np.zeros((2, 2), np.complex64)),
                            "ad", ctx=ctx)
    assert e.value.status == 2
    # The context stays usable.
    B = np.ones((3, 2), np.complex64)
    C = np.zeros((2, 2), np.complex64)
    t1m.contract_scaled(1.0, t1m.tensor.from_array(np.ones((2, 3), np.complex64)), "ab",
                        t1m.tensor.from_array(B), "bc", 0.0, t1m.tensor.from_array(C), "ac",
                        ctx=ctx)
    assert np.allclose(C, 3.0)
