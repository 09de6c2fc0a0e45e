"""Real float32 contractions on the tensor cores (the 3xTF32 / BF16x3 / BF16x6
split methods without the 1M expansion) against the FP64 oracle and the
reference's outputs (gpu)."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import numpy_oracle as no

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
FIX = np.load(GOLDEN / "contractions.npz")
F32_KEYS = sorted({k.rsplit("__", 1)[0] for k in FIX.files if "__f32__" in k})

TOL = {"tc_3xtf32": 1e-6, "tc_bf16x6": 1e-6, "tc_bf16x3": 2e-5, "auto": 1e-6}
# Row-major 2-D operands; the last label of each is its unit-stride mode,
# which selects the fetch modes (A [k][m] / [m][k], B [n][k] / [k][n]).
COMBOS = [("mk", "kn", "mn"), ("mk", "kn", "nm"), ("mk", "nk", "mn"), ("km", "kn", "mn"),
          ("km", "nk", "mn"), ("km", "nk", "nm")]


def _mats(la, lb, X, Y):
    A = X if la == "mk" else X.T
    B = Y if lb == "kn" else Y.T
    return A.astype(np.float64), B.astype(np.float64)


@pytest.mark.parametrize("method", ["tc_3xtf32", "tc_bf16x6", "tc_bf16x3", "auto"])
@pytest.mark.parametrize("combo", range(len(COMBOS)))
def test_real_tc_fetch_modes(ctx, torch_cuda, combo, method):
    import t1m_gb300 as t1m
    torch = torch_cuda
    la, lb, lc = COMBOS[combo]
    S = 1024
    rng = np.random.default_rng(80 + combo)
    Xh = rng.uniform(-1, 1, (S, S)).astype(np.float32)
    Yh = rng.uniform(-1, 1, (S, S)).astype(np.float32)
    X, Y = torch.from_numpy(Xh).cuda(), torch.from_numpy(Yh).cuda()
    C = torch.zeros((S, S), dtype=torch.float32, device="cuda")
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    ctx.set_method(method)
    try:
        outs = []
        for _ in range(3):
            rep = t1m.contract_scaled(1.0, v(X), la, v(Y), lb, 0.0, v(C), lc, ctx=ctx)
            torch.cuda.synchronize()
            outs.append(C.cpu().numpy())
    finally:
        ctx.set_method("auto")
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])   # no race between runs
    A, B = _mats(la, lb, Xh, Yh)
    ref = A @ B
    got = outs[0] if lc == "mn" else outs[0].T
    mx, fro = no.rel_errors(got.astype(np.float64), ref)
    assert mx < TOL[method] and fro < TOL[method], (method, mx, fro)
    assert rep.method in (2, 3, 4)   # a tensor-core method ran


@pytest.mark.parametrize("splits", [1, 3])
def test_real_tc_ragged_gathered_split(ctx, torch_cuda, splits):
    """Ragged extents, strided (gathered) operands, alpha/beta, forced split-K."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(90)
    A = rng.uniform(-1, 1, (7, 29, 11, 3)).astype(np.float32)     # a b c d
    B = rng.uniform(-1, 1, (11, 3, 13, 17)).astype(np.float32)    # c d e f
    C0 = rng.uniform(-1, 1, (29, 7, 17, 13)).astype(np.float32)   # b a f e
    ga, gb, gc = (torch.from_numpy(x.copy()).cuda() for x in (A, B, C0))
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    ctx.set_method("tc_3xtf32")
    ctx.set_split_k(splits)
    try:
        rep = t1m.contract_scaled(1.5, v(ga), "abcd", v(gb), "cdef", -0.5, v(gc), "bafe", ctx=ctx)
        torch.cuda.synchronize()
    finally:
        ctx.set_split_k(0)
        ctx.set_method("auto")
    ref = 1.5 * np.einsum("abcd,cdef->bafe", A.astype(np.float64), B.astype(np.float64)) \
        - 0.5 * C0.astype(np.float64)
    mx, fro = no.rel_errors(gc.cpu().numpy().astype(np.float64), ref)
    assert mx < 1e-6 and fro < 1e-6, (mx, fro)
    # K = 33 is two 32-element K steps: a forced split is capped at that.
    assert rep.method == 2 and (rep.split_k > 1) == (splits > 1)


@pytest.mark.parametrize("method", ["tc_3xtf32", "tc_bf16x6"])
@pytest.mark.parametrize("key", F32_KEYS)
def test_real_tc_reference_fixtures(ctx, key, method):
    """C += alpha*A*B on the committed seeded inputs equals the reference's output."""
    import t1m_gb300 as t1m
    meta = json.loads(str(FIX[key + "__meta"]))
    fa, fb, fc0, fc = (FIX[key + s] for s in ("__a", "__b", "__c0", "__c"))
    (la, lb, lc), (da, db, dc) = meta["labels"], meta["dims"]
    L = t1m.col_major if meta["layout"] == "col" else t1m.row_major
    ctx.set_method(method)
    try:
        c = fc0.copy()
        t1m.contract(meta["alpha"], t1m.tensor(da, fa, L), la, t1m.tensor(db, fb, L), lb, 0.0,
                     t1m.tensor(dc, c, L), lc, ctx=ctx)
    finally:
        ctx.set_method("auto")
    err = np.abs(c.astype(np.float64) - fc.astype(np.float64)).max() / max(np.abs(fc).max(), 1e-30)
    assert err < 2e-5, (method, err)
