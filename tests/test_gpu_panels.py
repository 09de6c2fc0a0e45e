"""B panels: products with at least four M tiles split B once (split_b_panels)
and load its pieces by TMA -- with 3xTF32, and with every method where B
would otherwise be gathered; smaller products split B inside the
tensor-core kernel.  The pieces and their K order are the same, so a product
computed whole (panels) and in slices of one M tile each (no panels) must
agree bit for bit, and both must meet the methods' accuracy against FP64
(gpu)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _one_tile_form(ctx):
    """Panels feed the one-tile-per-CTA kernel; where both operands load by
    TMA the automatic form runs CTA pairs instead (B split in-kernel)."""
    ctx.set_tile_form("one")
    yield
    ctx.set_tile_form("auto")

TOL = {"tc_3xtf32": 1e-6, "tc_bf16x6": 1e-6, "tc_bf16x3": 2e-5}


def _crand(rng, shape):
    return (rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(np.complex64)


def _whole_and_sliced(ctx, t1m, torch, A, la, B, lb, C0, lc, rows, conj_b=False, alpha=1.0,
                      beta=0.0):
    """C computed whole and in slices of `rows` along the leading (M) mode of
    A and C (row-major, so every slice is contiguous)."""
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    ga, gb = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    whole = torch.from_numpy(C0.copy()).cuda()
    rep = t1m.contract_scaled(alpha, v(ga), la, v(gb), lb, beta, v(whole), lc, ctx=ctx,
                              conj_b=conj_b)
    sliced = torch.from_numpy(C0.copy()).cuda()
    reps = []
    for m0 in range(0, A.shape[0], rows):
        a, c = ga[m0:m0 + rows], sliced[m0:m0 + rows]
        reps.append(t1m.contract_scaled(alpha, v(a), la, v(gb), lb, beta, v(c), lc, ctx=ctx,
                                        conj_b=conj_b))
    torch.cuda.synchronize()
    return rep, reps, whole.cpu().numpy(), sliced.cpu().numpy()


@pytest.mark.parametrize("method", ["tc_3xtf32", "tc_bf16x6", "tc_bf16x3"])
@pytest.mark.parametrize("blayout", ["kn", "nk"])
def test_panels_bit_identical_complex(ctx, torch_cuda, method, blayout):
    """complex64 M = 320 (5 tiles), N = 200, K = 1000 (ragged), conj(B),
    alpha/beta; B [k][n] or [n][k]."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(120)
    M, N, K = 320, 200, 1000
    A = _crand(rng, (M, K))
    B = _crand(rng, (K, N) if blayout == "kn" else (N, K))
    C0 = _crand(rng, (M, N))
    ctx.set_method(method)
    ctx.set_split_k(1)   # no automatic split-K: one product kernel each
    try:
        rep, reps, whole, sliced = _whole_and_sliced(ctx, t1m, torch, A, "mk", B, blayout, C0,
                                                     "mn", 64, conj_b=True, alpha=0.5 - 1j,
                                                     beta=0.25)
    finally:
        ctx.set_split_k(0)
        ctx.set_method("auto")
    # Panel pass + product for 3xTF32; the bf16 methods split a TMA-loaded B
    # in the kernel.
    assert rep.kernels == (2 if method == "tc_3xtf32" else 1)
    assert all(r.kernels == 1 for r in reps)
    np.testing.assert_array_equal(whole, sliced)
    Bm = B.astype(np.complex128) if blayout == "kn" else B.T.astype(np.complex128)
    ref = (0.5 - 1j) * (A.astype(np.complex128) @ np.conj(Bm)) + 0.25 * C0
    err = np.abs(whole - ref).max() / np.abs(ref).max()
    assert err < TOL[method], err


@pytest.mark.parametrize("method", ["tc_3xtf32", "tc_bf16x6", "tc_bf16x3"])
def test_panels_gathered_b(ctx, torch_cuda, method):
    """B 'dfce' with K = (c, d) and N = (f, e) interleaved: no uniform 2-D
    view, so the panel pass gathers through the scatter vectors."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(121)
    Mx, c, d, e, f = 256, 24, 20, 12, 11
    A = _crand(rng, (Mx, c, d))
    B = _crand(rng, (d, f, c, e))
    C0 = np.zeros((Mx, e, f), np.complex64)
    ctx.set_method(method)
    ctx.set_split_k(1)   # no automatic split-K: one product kernel each
    try:
        rep, reps, whole, sliced = _whole_and_sliced(ctx, t1m, torch, A, "mcd", B, "dfce", C0,
                                                     "mef", 64)
    finally:
        ctx.set_split_k(0)
        ctx.set_method("auto")
    assert rep.kernels == 2
    np.testing.assert_array_equal(whole, sliced)
    ref = np.einsum("mcd,dfce->mef", A.astype(np.complex128), B.astype(np.complex128))
    err = np.abs(whole - ref).max() / np.abs(ref).max()
    assert err < TOL[method], err


def test_panels_split_k(ctx, torch_cuda):
    """Forced split-K: each split reads its own stages of the panels."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(122)
    M, N, K = 256, 256, 2048
    A, B = _crand(rng, (M, K)), _crand(rng, (K, N))
    C0 = np.zeros((M, N), np.complex64)
    ctx.set_method("tc_3xtf32")
    ctx.set_split_k(3)
    try:
        rep, reps, whole, sliced = _whole_and_sliced(ctx, t1m, torch, A, "mk", B, "kn", C0, "mn", 64)
    finally:
        ctx.set_split_k(0)
        ctx.set_method("auto")
    assert rep.split_k == 3 and rep.kernels == 3   # panels, product, reduction
    np.testing.assert_array_equal(whole, sliced)
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    assert np.abs(whole - ref).max() / np.abs(ref).max() < 1e-6


@pytest.mark.parametrize("method", ["tc_3xtf32", "tc_bf16x6", "tc_bf16x3"])
@pytest.mark.parametrize("blayout", ["kn", "nk"])
def test_panels_bit_identical_real(ctx, torch_cuda, method, blayout):
    """float32 M = 640 (5 tiles of 128 rows), N = 300, K = 776 (ragged against
    the 32-value stage; rows of B stay 16-byte aligned, so B is TMA-loaded)."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(123)
    M, N, K = 640, 300, 776
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N) if blayout == "kn" else (N, K)).astype(np.float32)
    C0 = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    ctx.set_method(method)
    ctx.set_split_k(1)   # no automatic split-K: one product kernel each
    try:
        rep, reps, whole, sliced = _whole_and_sliced(ctx, t1m, torch, A, "mk", B, blayout, C0,
                                                     "mn", 128, alpha=1.5, beta=-0.5)
    finally:
        ctx.set_split_k(0)
        ctx.set_method("auto")
    assert rep.kernels == (2 if method == "tc_3xtf32" else 1)
    assert all(r.kernels == 1 for r in reps)
    np.testing.assert_array_equal(whole, sliced)
    Bm = B.astype(np.float64) if blayout == "kn" else B.T.astype(np.float64)
    ref = 1.5 * (A.astype(np.float64) @ Bm) - 0.5 * C0
    err = np.abs(whole - ref).max() / np.abs(ref).max()
    assert err < TOL[method], err


@pytest.mark.parametrize("method", ["tc_3xtf32", "tc_bf16x6", "tc_bf16x3"])
def test_panels_gathered_b_real(ctx, torch_cuda, method):
    """float32 B 'dfce' (K = (c, d), N = (f, e) interleaved): gathered by
    the panel pass for every method."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(124)
    Mx, c, d, e, f = 512, 24, 20, 12, 11
    A = rng.uniform(-1, 1, (Mx, c, d)).astype(np.float32)
    B = rng.uniform(-1, 1, (d, f, c, e)).astype(np.float32)
    C0 = np.zeros((Mx, e, f), np.float32)
    ctx.set_method(method)
    ctx.set_split_k(1)
    try:
        rep, reps, whole, sliced = _whole_and_sliced(ctx, t1m, torch, A, "mcd", B, "dfce", C0,
                                                     "mef", 128)
    finally:
        ctx.set_split_k(0)
        ctx.set_method("auto")
    assert rep.kernels == 2
    np.testing.assert_array_equal(whole, sliced)
    ref = np.einsum("mcd,dfce->mef", A.astype(np.float64), B.astype(np.float64))
    err = np.abs(whole - ref).max() / np.abs(ref).max()
    assert err < TOL[method], err
