"""Host operands of large contractions run as a slab pipeline (copies of slab
i+1 / i-1 overlap the kernels of slab i).  Slabs are multiples of the kernels'
output tiles, so every output element is computed by the same arithmetic as
with device operands: the results must be identical (gpu)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rand(rng, n, dt):
    return (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(dt)


@pytest.mark.parametrize("method", ["tc_3xtf32", "tc_bf16x6", "plain"])
@pytest.mark.parametrize("layout", ["col", "row"])
@pytest.mark.parametrize("beta", [0.0, 0.25])
def test_pipelined_host_equals_device(ctx, torch_cuda, layout, method, beta):
    """ijkl,klmn->ijmn, extents 48 (A, B, C 42 MB each): slabs along N for
    col-major, along M for row-major; beta != 0 also streams C in.  BF16x6
    runs as operand pieces: the resident operand split once for all slabs."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    dims = [48] * 4
    n = 48 ** 4
    rng = np.random.default_rng(60)
    A, B, C0 = _rand(rng, n, np.complex64), _rand(rng, n, np.complex64), _rand(rng, n, np.complex64)
    L = t1m.col_major if layout == "col" else t1m.row_major
    alpha = 1 - 0.5j
    ctx.set_method(method)
    try:
        ch = C0.copy()
        rep = t1m.contract_scaled(alpha, t1m.tensor(dims, A, L), "ijkl", t1m.tensor(dims, B, L),
                                  "klmn", beta, t1m.tensor(dims, ch, L), "ijmn", ctx=ctx)
        ga, gb = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
        gc = torch.from_numpy(C0.copy()).cuda()
        t1m.contract_scaled(alpha, t1m.tensor(dims, ga, L), "ijkl", t1m.tensor(dims, gb, L),
                            "klmn", beta, t1m.tensor(dims, gc, L), "ijmn", ctx=ctx)
        torch.cuda.synchronize()
    finally:
        ctx.set_method("auto")
    assert rep.kernels >= 2  # one product per slab
    assert rep.h2d_bytes >= 2 * n * 8 and rep.d2h_bytes == n * 8
    if method == "tc_bf16x6":
        assert rep.fetch["pieces"], rep.fetch
    np.testing.assert_array_equal(ch, gc.cpu().numpy())


def test_pipelined_strided_c_keeps_gaps(ctx, torch_cuda):
    """C is a view with gaps (3000 of 3100 columns of a row-major array): the
    gap columns survive the slab copies unchanged."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(61)
    M = N = K = 3000
    A = _rand(rng, M * K, np.complex64).reshape(M, K)
    B = _rand(rng, K * N, np.complex64).reshape(K, N)
    big = _rand(rng, M * 3100, np.complex64).reshape(M, 3100)
    before = big.copy()
    Cv = big[:, :N]
    rep = t1m.contract_scaled(1.0, t1m.tensor.from_array(A), "ik", t1m.tensor.from_array(B), "kj",
                              0.0, t1m.tensor.from_array(Cv), "ij", ctx=ctx)
    assert rep.kernels >= 2
    np.testing.assert_array_equal(big[:, N:], before[:, N:])
    ga, gb = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    gc = torch.zeros((M, N), dtype=torch.complex64, device="cuda")
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    t1m.contract_scaled(1.0, v(ga), "ik", v(gb), "kj", 0.0, v(gc), "ij", ctx=ctx)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(Cv, gc.cpu().numpy())


@pytest.mark.parametrize("method", ["tc_3xtf32", "tc_bf16x6"])
def test_pipelined_narrow_last_slab(ctx, torch_cuda, method):
    """Row-major M = 2624, N = 1024, K = 6144: four slabs along M of 768 rows
    (96 tiles: the pipeline runs), the last 320 rows (40 tiles), each slab in
    two halves of B along N on alternating compute streams.  The last slab's
    blocks would split K on their own; pipeline blocks never split, so they
    stay bit-identical to the device path and never share the split-K
    workspace."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(62)
    M, N, K = 2624, 1024, 6144
    A = _rand(rng, M * K, np.complex64).reshape(M, K)
    B = _rand(rng, K * N, np.complex64).reshape(K, N)
    C = np.zeros((M, N), np.complex64)
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    ctx.set_method(method)
    try:
        rep = t1m.contract_scaled(1.0, v(A), "mk", v(B), "kn", 0.0, v(C), "mn", ctx=ctx)
        ga, gb = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
        gc = torch.zeros((M, N), dtype=torch.complex64, device="cuda")
        dev = t1m.contract_scaled(1.0, v(ga), "mk", v(gb), "kn", 0.0, v(gc), "mn", ctx=ctx)
        torch.cuda.synchronize()
    finally:
        ctx.set_method("auto")
    # 4 slabs x 2 halves (plus a panel pass per block for 3xTF32).
    assert rep.kernels >= 8 and rep.split_k == 1 and dev.split_k == 1, rep.kernels
    assert rep.h2d_bytes >= A.nbytes + B.nbytes and rep.d2h_bytes == C.nbytes
    np.testing.assert_array_equal(C, gc.cpu().numpy())
