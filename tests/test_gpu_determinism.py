"""Repeated tensor-core contractions give bit-identical results, in every
operand fetch-mode combination (gpu).

A tensor-core result can only change between identical runs through a data
race inside the kernel (the arithmetic and its order are fixed), so eight runs
of each combination must agree bit for bit, and with sampled FP64.  This
guards the pipeline's cross-proxy ordering: raw stages read by the converter
warps (generic proxy) and refilled by TMA (async proxy) — a missing fence
there showed as rows of C computed from the next stage's data."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

S = 2304
# (A labels, B labels, C labels) of row-major 2-D tensors; the last label of
# each is its unit-stride mode, which selects the fetch modes.
COMBOS = [("mk", "kn", "mn"),   # A [m][k] swizzled (K unit), B [k][n] (N unit), C pairs
          ("mk", "kn", "nm"),   # same operands, C written element by element
          ("mk", "nk", "mn"),   # A K unit, B [n][k] swizzled (K unit)
          ("km", "kn", "mn"),   # A [k][m] (M unit), B N unit
          ("km", "nk", "mn"),
          ("km", "nk", "nm")]


@pytest.mark.parametrize("method", ["tc_3xtf32", "tc_bf16x6", "tc_bf16x3"])
@pytest.mark.parametrize("combo", range(len(COMBOS)))
def test_repeated_runs_bit_identical(ctx, torch_cuda, combo, method):
    import t1m_gb300 as t1m
    torch = torch_cuda
    la, lb, lc = COMBOS[combo]
    rng = np.random.default_rng(70)
    Xh = (rng.uniform(-1, 1, (S, S)) + 1j * rng.uniform(-1, 1, (S, S))).astype(np.complex64)
    Yh = (rng.uniform(-1, 1, (S, S)) + 1j * rng.uniform(-1, 1, (S, S))).astype(np.complex64)
    X, Y = torch.from_numpy(Xh).cuda(), torch.from_numpy(Yh).cuda()
    C = torch.zeros((S, S), dtype=torch.complex64, device="cuda")
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    ctx.set_method(method)
    try:
        outs = []
        for _ in range(8):
            t1m.contract_scaled(1.0, v(X), la, v(Y), lb, 0.0, v(C), lc, ctx=ctx)
            torch.cuda.synchronize()
            outs.append(C.cpu().numpy())
    finally:
        ctx.set_method("auto")
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])
    A = Xh.astype(np.complex128) if la == "mk" else Xh.T.astype(np.complex128)
    B = Yh.astype(np.complex128) if lb == "kn" else Yh.T.astype(np.complex128)
    r = np.random.default_rng(0)
    ms, ns = r.integers(0, S, 256), r.integers(0, S, 256)
    want = np.einsum("sk,sk->s", A[ms], B[:, ns].T)
    got = outs[0][ms, ns] if lc == "mn" else outs[0][ns, ms]
    err = np.abs(got - want).max() / np.abs(want).max()
    assert err < (2e-5 if method == "tc_bf16x3" else 1e-6), err
