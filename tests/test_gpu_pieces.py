"""CTA pairs over operands split into bf16 pieces beforehand (gpu).

T1M_TILE_PIECES splits A (the 1M rows) and B once into bf16 pieces in the
workspace and runs the pair kernel with both MMA operands in shared memory.
Per accumulator its MMAs run in the in-kernel-split pair form's order, so the
two forms must agree bit for bit; both are also checked against FP64.  Cases:
every TMA operand layout pair, ragged M, N and K (a pair whose second CTA
holds no valid row, a last K stage past K), conjugation, complex alpha/beta,
split-K with K ranges of whole and half stages, and the fallback when the
workspace limit leaves no room for the pieces."""
import numpy as np
import pytest

from oracle import numpy_oracle as no

pytestmark = pytest.mark.gpu

METHODS = ["tc_bf16x6", "tc_bf16x3"]
TOL = {"tc_bf16x6": 1e-6, "tc_bf16x3": 2e-5}

CASES = [
    (("mk", "kn", "mn"), dict(m=512, k=512, n=384), "col"),
    (("mk", "kn", "mn"), dict(m=512, k=256, n=256), "row"),
    (("km", "kn", "mn"), dict(m=384, k=320, n=256), "col"),
    (("mk", "nk", "mn"), dict(m=256, k=320, n=256), "col"),
    (("mk", "kn", "mn"), dict(m=200, k=272, n=136), "col"),   # ragged M, N, K
    (("mk", "kn", "mn"), dict(m=64 * 3, k=100, n=128), "col"),  # 2nd CTA past M, K % 4 != 0
]


def _rand(rng, n):
    return (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)


def _run(ctx, torch, form, method, labels, dims, layout, fa, fb, fc0, alpha, beta, flags=0):
    import t1m_gb300 as t1m
    L = t1m.col_major if layout == "col" else t1m.row_major
    ctx.set_tile_form(form)
    ctx.set_method(method)
    ga, gb = torch.from_numpy(fa).cuda(), torch.from_numpy(fb).cuda()
    gc = torch.from_numpy(fc0.copy()).cuda()
    (la, lb, lc), (da, db, dc) = labels, dims
    rep = t1m.contract_raw(alpha, t1m.tensor(da, ga, L), la, t1m.tensor(db, gb, L), lb, beta,
                           t1m.tensor(dc, gc, L), lc, flags, ctx)
    torch.cuda.synchronize()
    return gc.cpu().numpy(), rep


def _both(ctx, torch, method, labels, dims, layout, fa, fb, fc0, alpha, beta, flags=0):
    try:
        pair, rp = _run(ctx, torch, "pair", method, labels, dims, layout, fa, fb, fc0, alpha,
                        beta, flags)
        pieces, rq = _run(ctx, torch, "pieces", method, labels, dims, layout, fa, fb, fc0, alpha,
                          beta, flags)
    finally:
        ctx.set_tile_form("auto")
        ctx.set_method("auto")
    return pair, rp, pieces, rq


def _fp64(fa, fb, fc0, dims, labels, layout, alpha, beta):
    st = no.col_major_strides if layout == "col" else no.row_major_strides
    views = [no.as_strided_view(f, d, st(d)) for f, d in zip((fa, fb, fc0), dims)]
    return no.contract_fp64(views[0], labels[0], views[1], labels[1], views[2], labels[2],
                            alpha, beta), st


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{','.join(c[0])}-{c[2]}-{c[1]['m']}")
def test_pieces_equal_pair_and_fp64(ctx, torch_cuda, case, method):
    torch = torch_cuda
    labels, ext, layout = case
    dims = [[ext[ch] for ch in s] for s in labels]
    rng = np.random.default_rng(51)
    fa, fb = _rand(rng, int(np.prod(dims[0]))), _rand(rng, int(np.prod(dims[1])))
    fc0 = _rand(rng, int(np.prod(dims[2])))
    alpha, beta = 1 + 0.5j, 0.25
    pair, rp, pieces, rq = _both(ctx, torch, method, labels, dims, layout, fa, fb, fc0, alpha,
                                 beta)
    assert rp.fetch["pair"] and not rp.fetch["pieces"], rp.fetch
    assert rq.fetch["pair"] and rq.fetch["pieces"], rq.fetch
    assert rq.kernels == rp.kernels + 1  # the split pass
    assert np.array_equal(pair.view(np.uint64), pieces.view(np.uint64))
    ref, st = _fp64(fa, fb, fc0, dims, labels, layout, alpha, beta)
    got = no.as_strided_view(pieces, dims[2], st(dims[2]))
    assert no.rel_errors(got, ref)[0] < TOL[method]


@pytest.mark.parametrize("flags", [2, 4, 6], ids=["conjA", "conjB", "conjAB"])
def test_pieces_conjugation(ctx, torch_cuda, flags):
    torch = torch_cuda
    labels, ext = ("mk", "kn", "mn"), dict(m=256, k=192, n=256)
    dims = [[ext[ch] for ch in s] for s in labels]
    rng = np.random.default_rng(52)
    fa, fb = _rand(rng, int(np.prod(dims[0]))), _rand(rng, int(np.prod(dims[1])))
    fc0 = np.zeros(int(np.prod(dims[2])), np.complex64)
    pair, _, pieces, rq = _both(ctx, torch, "tc_bf16x6", labels, dims, "col", fa, fb, fc0, 1.0,
                                0.0, flags)
    assert rq.fetch["pieces"]
    assert np.array_equal(pair.view(np.uint64), pieces.view(np.uint64))
    A = fa.reshape(dims[0], order="F")
    B = fb.reshape(dims[1], order="F")
    A = np.conj(A) if flags & 2 else A
    B = np.conj(B) if flags & 4 else B
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    assert no.rel_errors(pieces.reshape(dims[2], order="F"), ref)[0] < 1e-6


@pytest.mark.parametrize("splits", [5, 3])
def test_pieces_split_k(ctx, torch_cuda, splits):
    """Forced split-K: 5 splits of K = 2048 give 416 complex k per split (a
    whole number of the pieces form's 32-k stages), 3 give 688 (each split
    ends half way through a stage).  Equal to the pair form's split result."""
    torch = torch_cuda
    labels, ext = ("mk", "kn", "mn"), dict(m=256, k=2048, n=128)
    dims = [[ext[ch] for ch in s] for s in labels]
    rng = np.random.default_rng(53)
    fa, fb = _rand(rng, int(np.prod(dims[0]))), _rand(rng, int(np.prod(dims[1])))
    fc0 = _rand(rng, int(np.prod(dims[2])))
    ctx.set_split_k(splits)
    try:
        pair, _, pieces, rq = _both(ctx, torch, "tc_bf16x6", labels, dims, "col", fa, fb, fc0,
                                    0.5, 1.0)
    finally:
        ctx.set_split_k(0)
    assert rq.split_k == splits and rq.fetch["pair"] and rq.fetch["pieces"]
    assert np.array_equal(pair.view(np.uint64), pieces.view(np.uint64))
    ref, _ = _fp64(fa, fb, fc0, dims, labels, "col", 0.5, 1.0)
    assert no.rel_errors(pieces.reshape(dims[2], order="F"), ref)[0] < 1e-6


def test_pieces_without_workspace(ctx, torch_cuda):
    """A workspace limit below the pieces' bytes: the product runs as plain
    pairs, with the same result."""
    torch = torch_cuda
    labels, ext = ("mk", "kn", "mn"), dict(m=512, k=512, n=256)
    dims = [[ext[ch] for ch in s] for s in labels]
    rng = np.random.default_rng(54)
    fa, fb = _rand(rng, int(np.prod(dims[0]))), _rand(rng, int(np.prod(dims[1])))
    fc0 = np.zeros(int(np.prod(dims[2])), np.complex64)
    ctx.set_workspace_limit(1 << 20)
    try:
        pair, _, pieces, rq = _both(ctx, torch, "tc_bf16x6", labels, dims, "col", fa, fb, fc0,
                                    1.0, 0.0)
    finally:
        ctx.set_workspace_limit(-1)
    assert rq.fetch["pair"] and not rq.fetch["pieces"]
    assert np.array_equal(pair.view(np.uint64), pieces.view(np.uint64))


@pytest.mark.parametrize("layout", ["col", "row"])
def test_pieces_host_pipeline(ctx, torch_cuda, layout):
    """Host operands (slab pipeline, slabs along N for col-major and along M
    for row-major): the resident operand is split into pieces once, each
    block splits only its streamed slab.  Equal to the device-buffer result
    and to the pair form's, bit for bit."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    dims = [48] * 4
    n = 48 ** 4
    rng = np.random.default_rng(55)
    A, B = _rand(rng, n), _rand(rng, n)
    L = t1m.col_major if layout == "col" else t1m.row_major
    out = {}
    ctx.set_method("tc_bf16x6")
    try:
        for form in ("pieces", "pair"):
            ctx.set_tile_form(form)
            ch = np.zeros(n, np.complex64)
            rep = t1m.contract_scaled(1.0, t1m.tensor(dims, A, L), "ijkl", t1m.tensor(dims, B, L),
                                      "klmn", 0.0, t1m.tensor(dims, ch, L), "ijmn", ctx=ctx)
            out[form] = (ch, rep)
        ctx.set_tile_form("pieces")
        ga, gb = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
        gc = torch.zeros(n, dtype=torch.complex64, device="cuda")
        dev = t1m.contract_scaled(1.0, t1m.tensor(dims, ga, L), "ijkl", t1m.tensor(dims, gb, L),
                                  "klmn", 0.0, t1m.tensor(dims, gc, L), "ijmn", ctx=ctx)
        torch.cuda.synchronize()
    finally:
        ctx.set_tile_form("auto")
        ctx.set_method("auto")
    ch, rep = out["pieces"]
    assert rep.h2d_bytes >= 2 * n * 8 and rep.fetch["pieces"] and dev.fetch["pieces"]
    assert not out["pair"][1].fetch["pieces"]
    np.testing.assert_array_equal(ch, gc.cpu().numpy())
    np.testing.assert_array_equal(ch, out["pair"][0])
