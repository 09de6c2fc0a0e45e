"""CTA pairs (tcgen05 cta_group::2) against the one-tile-per-CTA form (gpu).

The pair form runs the same split products in the same K order, with one MMA
of 256 x 128 real rows per pair instead of two of 128 x 128, so its results
must equal the one-tile form's bit for bit; both are also checked against
FP64.  Cases cover every TMA operand layout pair ([k][m] / [m][k] A, [n][k] /
[k][n] B), the three split methods, ragged M and N (a pair whose second CTA
holds no valid row), conjugation, complex alpha/beta and split-K."""
import numpy as np
import pytest

from oracle import numpy_oracle as no

pytestmark = pytest.mark.gpu

METHODS = ["tc_bf16x6", "tc_3xtf32", "tc_bf16x3"]
TOL = {"tc_bf16x6": 1e-6, "tc_3xtf32": 1e-6, "tc_bf16x3": 2e-5}

# (labels, extents, layout): col-major mk,kn gives A [k][m] and B [n][k];
# row-major the transposes; the km/nk label orders give the mixed pairs.
CASES = [
    (("mk", "kn", "mn"), dict(m=512, k=512, n=384), "col"),
    (("mk", "kn", "mn"), dict(m=512, k=256, n=256), "row"),
    (("km", "kn", "mn"), dict(m=384, k=320, n=256), "col"),
    (("mk", "nk", "mn"), dict(m=256, k=320, n=256), "col"),
    (("mk", "kn", "mn"), dict(m=200, k=272, n=136), "col"),   # ragged M and N
    (("mk", "kn", "mn"), dict(m=64 * 3, k=128, n=128), "col"),  # 2nd CTA of a pair past M
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


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{','.join(c[0])}-{c[2]}-{c[1]['m']}")
def test_pair_equals_one_tile_and_fp64(ctx, torch_cuda, case, method):
    import t1m_gb300 as t1m
    torch = torch_cuda
    labels, ext, layout = case
    dims = [[ext[ch] for ch in s] for s in labels]
    rng = np.random.default_rng(31)
    fa, fb = _rand(rng, int(np.prod(dims[0]))), _rand(rng, int(np.prod(dims[1])))
    fc0 = _rand(rng, int(np.prod(dims[2])))
    alpha, beta = 1 + 0.5j, 0.25
    try:
        one, r1 = _run(ctx, torch, "one", method, labels, dims, layout, fa, fb, fc0, alpha, beta)
        two, r2 = _run(ctx, torch, "pair", method, labels, dims, layout, fa, fb, fc0, alpha, beta)
    finally:
        ctx.set_tile_form("auto")
        ctx.set_method("auto")
    assert r2.fetch["pair"] and not r1.fetch["pair"], (r1.fetch, r2.fetch)
    assert np.array_equal(one.view(np.uint64), two.view(np.uint64))
    st = no.col_major_strides if layout == "col" else no.row_major_strides
    views = [no.as_strided_view(f, d, st(d)) for f, d in zip((fa, fb, fc0), dims)]
    ref = no.contract_fp64(views[0], labels[0], views[1], labels[1], views[2], labels[2],
                           alpha, beta)
    got = no.as_strided_view(two, dims[2], st(dims[2]))
    assert no.rel_errors(got, ref)[0] < TOL[method]


@pytest.mark.parametrize("flags", [2, 4, 6], ids=["conjA", "conjB", "conjAB"])
def test_pair_conjugation(ctx, torch_cuda, flags):
    torch = torch_cuda
    labels, ext = ("mk", "kn", "mn"), dict(m=256, k=192, n=256)
    dims = [[ext[ch] for ch in s] for s in labels]
    rng = np.random.default_rng(32)
    fa, fb = _rand(rng, int(np.prod(dims[0]))), _rand(rng, int(np.prod(dims[1])))
    fc0 = np.zeros(int(np.prod(dims[2])), np.complex64)
    try:
        one, _ = _run(ctx, torch, "one", "tc_bf16x6", labels, dims, "col", fa, fb, fc0, 1.0, 0.0,
                      flags)
        two, rep = _run(ctx, torch, "pair", "tc_bf16x6", labels, dims, "col", fa, fb, fc0, 1.0,
                        0.0, flags)
    finally:
        ctx.set_tile_form("auto")
        ctx.set_method("auto")
    assert rep.fetch["pair"]
    assert np.array_equal(one.view(np.uint64), two.view(np.uint64))
    A = fa.reshape(dims[0], order="F")
    B = fb.reshape(dims[1], order="F")
    A = np.conj(A) if flags & 2 else A
    B = np.conj(B) if flags & 4 else B
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    got = two.reshape(dims[2], order="F")
    assert no.rel_errors(got, ref)[0] < 1e-6


def test_pair_split_k(ctx, torch_cuda):
    """Forced split-K through the pair form: raw partials per split, FP64
    reduction; equal to the one-tile form's split result."""
    torch = torch_cuda
    labels, ext = ("mk", "kn", "mn"), dict(m=256, k=2048, n=128)
    dims = [[ext[ch] for ch in s] for s in labels]
    rng = np.random.default_rng(33)
    fa, fb = _rand(rng, int(np.prod(dims[0]))), _rand(rng, int(np.prod(dims[1])))
    fc0 = _rand(rng, int(np.prod(dims[2])))
    ctx.set_split_k(5)
    try:
        one, _ = _run(ctx, torch, "one", "tc_3xtf32", labels, dims, "col", fa, fb, fc0, 0.5, 1.0)
        two, rep = _run(ctx, torch, "pair", "tc_3xtf32", labels, dims, "col", fa, fb, fc0, 0.5, 1.0)
    finally:
        ctx.set_split_k(0)
        ctx.set_tile_form("auto")
        ctx.set_method("auto")
    assert rep.split_k == 5 and rep.fetch["pair"]
    assert np.array_equal(one.view(np.uint64), two.view(np.uint64))
