"""The bf16 split-product tensor-core forms (t1m_method TC_BF16X3 and
TC_BF16X6) against the reference's outputs and the FP64 oracle (gpu).

Error budgets (normwise, max|dC| / max|C|), from the splits: a value x is
cut into bf16 pieces x0 + x1 (+ x2), each the round-to-nearest bf16 of the
remainder, so |x - x0| <= 2^-9 |x| and |x - x0 - x1| <= 2^-18 |x|.
  BF16x3 (x0y0 + x0y1 + x1y0) drops x1y1 and the second remainders:
         <= 3 * 2^-18 |x||y| per product, so 2e-5 against FP64 (measured
         3-4e-6 at K = 256..4096) and 5e-5 against the reference's FP32
         output at fixture sizes.
  BF16x6 (+ x1y1 + x0y2 + x2y0) leaves terms of 2^-27: an FP32-class result,
         held to the same 1e-6 bar as 3xTF32.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import numpy_oracle as no

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
FIX = np.load(GOLDEN / "contractions.npz")
C64_KEYS = sorted({k.rsplit("__", 1)[0] for k in FIX.files if "__c64__" in k})

BF16_METHODS = ["tc_bf16x3", "tc_bf16x6"]
TOL_FP64 = {"tc_bf16x3": 2e-5, "tc_bf16x6": 1e-6}
TOL_REF = {"tc_bf16x3": 5e-5, "tc_bf16x6": 2e-5}


def _fixture(key):
    meta = json.loads(str(FIX[key + "__meta"]))
    return meta, FIX[key + "__a"], FIX[key + "__b"], FIX[key + "__c0"], FIX[key + "__c"]


def _rand(rng, shape):
    return (rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(np.complex64)


@pytest.mark.parametrize("method", BF16_METHODS)
@pytest.mark.parametrize("key", C64_KEYS)
def test_bf16_reference_fixtures(ctx, key, method):
    """C += A*B on the committed seeded inputs equals the reference's output."""
    import t1m_gb300 as t1m
    meta, fa, fb, fc0, fc = _fixture(key)
    (la, lb, lc), (da, db, dc) = meta["labels"], meta["dims"]
    L = t1m.col_major if meta["layout"] == "col" else t1m.row_major
    ctx.set_method(method)
    try:
        c = fc0.copy()
        rep = t1m.contract(t1m.tensor(da, fa, L), la, t1m.tensor(db, fb, L), lb,
                           t1m.tensor(dc, c, L), lc, ctx=ctx)
    finally:
        ctx.set_method("auto")
    assert rep.method == t1m.method[method]
    scale = max(np.abs(fc).max(), 1e-30)
    err = np.abs(c.astype(np.complex128) - fc.astype(np.complex128)).max() / scale
    assert err < TOL_REF[method], (method, err)


# Every operand fetch path of the kernel: A [k][m] TMA (M unit stride) and
# B [n][k] TMA (K unit stride); A [m][k] / B [k][n] TMA (row-major); element
# gathers through the scatter vectors; ragged edges in M, N and K.
MODE_CASES = [
    ("mk", "kn", "mn", "col", dict(m=256, k=256, n=256)),
    ("mk", "kn", "mn", "row", dict(m=256, k=256, n=256)),
    ("abcd", "dbea", "ec", "col", dict(a=6, b=8, c=96, d=12, e=64)),
    ("km", "kn", "mn", "col", dict(m=200, k=144, n=136)),
    ("mk", "kn", "mn", "row", dict(m=70, k=37, n=130)),
]


@pytest.mark.parametrize("conj", [(False, False), (True, False), (False, True)])
@pytest.mark.parametrize("case", range(len(MODE_CASES)))
def test_bf16_fetch_modes_vs_fp64(ctx, torch_cuda, case, conj):
    import t1m_gb300 as t1m
    torch = torch_cuda
    la, lb, lc, layout, ext = MODE_CASES[case]
    da, db, dc = ([ext[ch] for ch in s] for s in (la, lb, lc))
    order = "F" if layout == "col" else "C"
    L = t1m.col_major if layout == "col" else t1m.row_major
    rng = np.random.default_rng(100 + case)
    A, B = _rand(rng, da), _rand(rng, db)
    Ar = np.conj(A) if conj[0] else A
    Br = np.conj(B) if conj[1] else B
    ref = np.einsum(f"{la},{lb}->{lc}", Ar.astype(np.complex128), Br.astype(np.complex128))
    errs = {}
    for m in BF16_METHODS:
        ctx.set_method(m)
        ga = torch.from_numpy(A.flatten(order=order)).cuda()
        gb = torch.from_numpy(B.flatten(order=order)).cuda()
        gc = torch.zeros(int(np.prod(dc)), dtype=torch.complex64, device="cuda")
        t1m.contract_scaled(1.0, t1m.tensor(da, ga, L), la, t1m.tensor(db, gb, L), lb, 0.0,
                            t1m.tensor(dc, gc, L), lc, ctx=ctx, conj_a=conj[0], conj_b=conj[1])
        torch.cuda.synchronize()
        got = gc.cpu().numpy().reshape(dc, order=order)
        mx, fro = no.rel_errors(got, ref)
        assert mx < TOL_FP64[m] and fro < TOL_FP64[m], (m, mx, fro)
        errs[m] = mx
    ctx.set_method("auto")
    # The three second-order products are what BF16x6 adds: it must be the
    # more accurate form.
    assert errs["tc_bf16x6"] < errs["tc_bf16x3"], errs


@pytest.mark.parametrize("splits", [2, 5])
def test_bf16_split_k(ctx, splits):
    """Forced split-K (FP64 reduction of partial products) with the bf16 forms."""
    import t1m_gb300 as t1m
    meta, fa, fb, fc0, fc = _fixture("cfg2b_small__c64__col")
    (la, lb, lc), (da, db, dc) = meta["labels"], meta["dims"]
    for m in BF16_METHODS:
        ctx.set_method(m)
        ctx.set_split_k(splits)
        try:
            c = fc0.copy()
            rep = t1m.contract(t1m.tensor(da, fa, t1m.col_major), la,
                               t1m.tensor(db, fb, t1m.col_major), lb,
                               t1m.tensor(dc, c, t1m.col_major), lc, ctx=ctx)
        finally:
            ctx.set_split_k(0)
            ctx.set_method("auto")
        assert rep.split_k > 1
        err = np.abs(c.astype(np.complex128) - fc.astype(np.complex128)).max() / np.abs(fc).max()
        assert err < TOL_REF[m], (m, err)


@pytest.mark.slow
@pytest.mark.parametrize("inputs", ["uniform", "logmag"])
def test_bf16_config3_full_size(ctx, torch_cuda, inputs):
    """complex64 ijkl,klmn->ijmn, extents 64 (M = N = K = 4096), both input
    sets: BF16x6 meets 1e-6 against sampled FP64, BF16x3 its 2e-5 budget."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    n = 4096 * 4096
    g = torch.Generator(device="cuda")
    g.manual_seed(21)

    def mk():
        if inputs == "uniform":
            return torch.complex(torch.rand(n, device="cuda", generator=g) * 2 - 1,
                                 torch.rand(n, device="cuda", generator=g) * 2 - 1)
        mag = torch.pow(10.0, torch.rand(n, device="cuda", generator=g) * 6 - 3)
        return torch.polar(mag, torch.rand(n, device="cuda", generator=g) * 2 * np.pi)

    ga, gb = mk(), mk()
    dims = [64] * 4
    fa, fb = ga.cpu().numpy(), gb.cpu().numpy()
    strides = no.col_major_strides(dims)
    scat = no.matricize("ijkl", "klmn", "ijmn", dims, dims, dims, strides, strides, strides)
    rng = np.random.default_rng(3)
    rows = rng.integers(0, 4096, 512)
    cols = rng.integers(0, 4096, 512)
    ref = no.sampled_entries(fa, fb, scat, rows, cols)
    off = scat[4][rows] + scat[5][cols]
    for m in BF16_METHODS:
        ctx.set_method(m)
        gc = torch.zeros(n, dtype=torch.complex64, device="cuda")
        rep = t1m.contract_scaled(1.0, t1m.tensor(dims, ga), "ijkl", t1m.tensor(dims, gb),
                                  "klmn", 0.0, t1m.tensor(dims, gc), "ijmn", ctx=ctx)
        torch.cuda.synchronize()
        got = gc.cpu().numpy()[off].astype(np.complex128)
        mx, fro = no.rel_errors(got, ref)
        assert mx < TOL_FP64[m] and fro < TOL_FP64[m], (m, inputs, mx, fro)
        assert rep.method == t1m.method[m]
    ctx.set_method("auto")
