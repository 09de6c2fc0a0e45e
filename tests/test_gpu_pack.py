"""Dense repack of gathered operands (pack.cu): an operand that the
tensor-core kernels would gather element by element, of 4 MB or more, is
packed into [rows][k] first and loaded by TMA.  The packed operand holds the
same values in the same K order, so a product computed whole (packed A) and
in slices of 8 rows (A below the size threshold, gathered) must agree bit for
bit under the same split-K, and both must meet 1e-6 against FP64 (gpu)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# The permuted drop-in case abcd,dbea->ec, column-major (A 28 MB, B 19 MB).
EXT = dict(a=24, b=32, c=96, d=48, e=64)


def _col_strides(dims):
    s, out = 1, []
    for d in dims:
        out.append(s)
        s *= d
    return out


def _operand(rng, labels, dt, ext=EXT):
    dims = [ext[ch] for ch in labels]
    n = int(np.prod(dims))
    if np.dtype(dt).kind == "c":
        flat = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(dt)
    else:
        flat = rng.uniform(-1, 1, n).astype(dt)
    return dims, flat


def _ref(la, lb, lc, fa, fb, da, db, dc):
    A = fa.astype(np.complex128 if fa.dtype.kind == "c" else np.float64).reshape(da[::-1]).T
    B = fb.astype(A.dtype).reshape(db[::-1]).T
    return np.einsum(f"{la},{lb}->{lc}", A, B)


def _run(ctx, t1m, torch, la, lb, lc, fa, fb, da, db, dc, slice_label, rows, ext=EXT):
    """C computed whole and in slices of `rows` of C's and A's `slice_label`
    mode (column-major tensors viewed with explicit strides)."""
    ga, gb = torch.from_numpy(fa).cuda(), torch.from_numpy(fb).cuda()
    sa, sb, sc = _col_strides(da), _col_strides(db), _col_strides(dc)
    nc = int(np.prod(dc))
    whole = torch.zeros(nc, dtype=ga.dtype, device="cuda")
    rep = t1m.contract_scaled(1.0, t1m.tensor(da, ga, t1m.STRIDED, sa), la,
                              t1m.tensor(db, gb, t1m.STRIDED, sb), lb, 0.0,
                              t1m.tensor(dc, whole, t1m.STRIDED, sc), lc, ctx=ctx)
    sliced = torch.zeros(nc, dtype=ga.dtype, device="cuda")
    ia, ic = la.index(slice_label), lc.index(slice_label)
    reps = []
    for r0 in range(0, ext[slice_label], rows):
        das, dcs = list(da), list(dc)
        das[ia] = dcs[ic] = rows
        a_view = ga[r0 * sa[ia]:]
        c_view = sliced[r0 * sc[ic]:]
        reps.append(t1m.contract_scaled(1.0, t1m.tensor(das, a_view, t1m.STRIDED, sa), la,
                                        t1m.tensor(db, gb, t1m.STRIDED, sb), lb, 0.0,
                                        t1m.tensor(dcs, c_view, t1m.STRIDED, sc), lc, ctx=ctx))
    torch.cuda.synchronize()
    return rep, reps, whole.cpu().numpy(), sliced.cpu().numpy()


@pytest.mark.parametrize("dt", [np.complex64, np.float32])
def test_pack_a_bit_identical(ctx, torch_cuda, dt):
    """abcd,dbea->ec: K follows B (d fastest), so A (unit stride along a) is
    gathered element by element; whole products pack it."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(130)
    la, lb, lc = "abcd", "dbea", "ec"
    da, fa = _operand(rng, la, dt)
    db, fb = _operand(rng, lb, dt)
    dc = [EXT[ch] for ch in lc]
    ctx.set_method("tc_3xtf32")
    ctx.set_split_k(8)
    try:
        rep, reps, whole, sliced = _run(ctx, t1m, torch, la, lb, lc, fa, fb, da, db, dc, "c", 8)
    finally:
        ctx.set_split_k(0)
        ctx.set_method("auto")
    # Whole: pack A, product, split-K reduction; slices: product, reduction.
    # float32 B has no per-block TMA form: it is packed in both.
    whole_k, slice_k = (3, 2) if dt == np.complex64 else (4, 3)
    assert rep.kernels == whole_k and all(r.kernels == slice_k for r in reps), (
        rep.kernels, [r.kernels for r in reps])
    np.testing.assert_array_equal(whole, sliced)
    ref = _ref(la, lb, lc, fa, fb, da, db, dc).T.reshape(-1)
    err = np.abs(whole - ref).max() / np.abs(ref).max()
    assert err < 1e-6, err


def test_pack_a_and_b(ctx, torch_cuda):
    """mqp,pnq->mn, column-major, p = 8: K follows B's unit-stride p, whose
    8-element runs leave neither operand with unit-stride 16-element K blocks,
    so both are gathered element by element and both are packed (A along its
    unit-stride rows, B elementwise).  Slices of 8 rows gather A and pack B."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    ext = dict(m=128, n=96, p=8, q=4096)
    rng = np.random.default_rng(131)
    la, lb, lc = "mqp", "pnq", "mn"
    da, fa = _operand(rng, la, np.complex64, ext)
    db, fb = _operand(rng, lb, np.complex64, ext)
    dc = [ext[ch] for ch in lc]
    ctx.set_method("tc_3xtf32")
    ctx.set_split_k(8)
    try:
        rep, reps, whole, sliced = _run(ctx, t1m, torch, la, lb, lc, fa, fb, da, db, dc, "m", 8,
                                        ext)
    finally:
        ctx.set_split_k(0)
        ctx.set_method("auto")
    assert rep.kernels == 4 and all(r.kernels == 3 for r in reps), (rep.kernels,
                                                                    [r.kernels for r in reps])
    np.testing.assert_array_equal(whole, sliced)
    ref = _ref(la, lb, lc, fa, fb, da, db, dc).T.reshape(-1)
    err = np.abs(whole - ref).max() / np.abs(ref).max()
    assert err < 1e-6, err


def test_pack_auto_config2b(ctx, torch_cuda):
    """The automatic method on abcd,dbea->ec packs A and meets 1e-6."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(132)
    la, lb, lc = "abcd", "dbea", "ec"
    da, fa = _operand(rng, la, np.complex64)
    db, fb = _operand(rng, lb, np.complex64)
    dc = [EXT[ch] for ch in lc]
    ga, gb = torch.from_numpy(fa).cuda(), torch.from_numpy(fb).cuda()
    gc = torch.zeros(int(np.prod(dc)), dtype=torch.complex64, device="cuda")
    rep = t1m.contract_scaled(1.0, t1m.tensor(da, ga, t1m.col_major), la,
                              t1m.tensor(db, gb, t1m.col_major), lb, 0.0,
                              t1m.tensor(dc, gc, t1m.col_major), lc, ctx=ctx)
    torch.cuda.synchronize()
    assert rep.method in (2, 4)
    ref = _ref(la, lb, lc, fa, fb, da, db, dc).T.reshape(-1)
    got = gc.cpu().numpy()
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 1e-6, err


def test_pack_block_mode_a(ctx, torch_cuda):
    """abcd,ebfd->aecf at extents 32 (the adjoint workload's product): A's
    per-16-row block form is packed so the product runs on the one-tile
    kernel with B from panels (pack, panel pass, product), and the automatic
    method meets 1e-6 against FP64."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    ext = dict(a=32, b=32, c=32, d=32, e=32, f=32)
    rng = np.random.default_rng(133)
    la, lb, lc = "abcd", "ebfd", "aecf"
    da, fa = _operand(rng, la, np.complex64, ext)
    db, fb = _operand(rng, lb, np.complex64, ext)
    dc = [ext[ch] for ch in lc]
    ga, gb = torch.from_numpy(fa).cuda(), torch.from_numpy(fb).cuda()
    gc = torch.zeros(int(np.prod(dc)), dtype=torch.complex64, device="cuda")
    rep = t1m.contract_scaled(1.0, t1m.tensor(da, ga, t1m.col_major), la,
                              t1m.tensor(db, gb, t1m.col_major), lb, 0.0,
                              t1m.tensor(dc, gc, t1m.col_major), lc, ctx=ctx)
    torch.cuda.synchronize()
    assert rep.kernels == 3, rep.kernels
    ref = _ref(la, lb, lc, fa, fb, da, db, dc).T.reshape(-1)
    got = gc.cpu().numpy()
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 1e-6, err
