"""Grouped batches (t1m_group_*): results equal the same contractions issued
one call at a time, and the FP64 oracle (gpu)."""
import numpy as np
import pytest

from oracle import numpy_oracle as no

pytestmark = pytest.mark.gpu


def _rand(rng, shape, dt, scale=1.0):
    x = rng.normal(0, scale, shape) + 1j * rng.normal(0, scale, shape)
    return x.astype(dt)


def _sweep_items(torch, t1m, rng, n, choices, st_choices, dt=np.complex64):
    """Config-4-style updates: xay,asb->xsyb then xsyb,ytb->xst."""
    items, host = [], []
    for _ in range(n):
        x, y, a, b = (int(v) for v in rng.choice(choices, 4))
        s, t = (int(v) for v in rng.choice(st_choices, 2))
        bond = np.sqrt(a)
        X1 = _rand(rng, (x, a, y), dt, 1 / np.sqrt(bond))
        X2 = _rand(rng, (a, s, b), dt, 1 / np.sqrt(bond))
        X3 = _rand(rng, (y, t, b), dt, 1 / np.sqrt(bond))
        g1, g2, g3 = (torch.from_numpy(v.copy()).cuda() for v in (X1, X2, X3))
        r1 = torch.zeros((x, s, y, b), dtype=g1.dtype, device="cuda")
        out = torch.zeros((x, s, t), dtype=g1.dtype, device="cuda")
        v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
        i1 = len(items)
        items.append((1.0, v(g1), "xay", v(g2), "asb", 0.0, v(r1), "xsyb", -1))
        items.append((1.0, v(r1), "xsyb", v(g3), "ytb", 0.0, v(out), "xst", i1))
        host.append((X1, X2, X3, r1, out, (g1, g2, g3)))
    return items, host


@pytest.mark.parametrize("graph", [True, False])
@pytest.mark.parametrize("autotune", [False, True])
def test_sweep_batch_matches_fp64(ctx, torch_cuda, graph, autotune, tmp_path, monkeypatch):
    import t1m_gb300 as t1m
    torch = torch_cuda
    monkeypatch.setenv("T1M_TUNE_CACHE", str(tmp_path / "tune.txt"))
    rng = np.random.default_rng(31)
    items, host = _sweep_items(torch, t1m, rng, 6, [16, 32, 48], [2, 4])
    grp = t1m.Group(items, ctx=ctx, graph=graph, autotune=autotune)
    for _ in range(2):  # relaunch (graph replay) gives the same result
        rep = grp.launch()
        assert rep.kernels >= 1
        for X1, X2, X3, r1, out, _ in host:
            R = np.einsum("xay,asb->xsyb", X1.astype(np.complex128), X2.astype(np.complex128))
            ref = np.einsum("xsyb,ytb->xst", R, X3.astype(np.complex128))
            for got, want in ((r1, R), (out, ref)):
                mx, fro = no.rel_errors(got.cpu().numpy(), want)
                assert mx < 2e-6 and fro < 2e-6, (mx, fro)
    grp.close()
    if autotune:
        assert (tmp_path / "tune.txt").exists()


def test_all_tensor_core_batch_with_dependencies(ctx, torch_cuda):
    """Every item on the tensor cores and two dependency levels: one
    persistent launch resolves the dependencies in the kernel (K of every
    item within the per-tile cap, so no item is split)."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(32)
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    items, checks = [], []
    for _ in range(5):
        x, a, q = (int(val) for val in rng.choice([32, 48, 64, 96], 3))
        y, b = (int(val) for val in rng.choice([16, 32], 2))
        X1 = _rand(rng, (x, a), np.complex64, 0.2)
        X2 = _rand(rng, (a, y, b), np.complex64, 0.2)
        X3 = _rand(rng, (y, b, q), np.complex64, 0.2)
        g1, g2, g3 = (torch.from_numpy(val.copy()).cuda() for val in (X1, X2, X3))
        r1 = torch.zeros((x, y, b), dtype=torch.complex64, device="cuda")
        out = torch.zeros((x, q), dtype=torch.complex64, device="cuda")
        i1 = len(items)
        items.append((1.0, v(g1), "xa", v(g2), "ayb", 0.0, v(r1), "xyb", -1))
        items.append((0.5j, v(r1), "xyb", v(g3), "ybq", 0.0, v(out), "xq", i1))
        checks.append((X1, X2, X3, r1, out, (g1, g2, g3)))
    grp = t1m.Group(items, ctx=ctx, graph=True)
    rep = grp.launch()
    assert rep.kernels == 1
    for X1, X2, X3, r1, out, _ in checks:
        R = np.einsum("xa,ayb->xyb", X1.astype(np.complex128), X2.astype(np.complex128))
        ref = 0.5j * np.einsum("xyb,ybq->xq", R, X3.astype(np.complex128))
        for got, want in ((r1, R), (out, ref)):
            mx, fro = no.rel_errors(got.cpu().numpy(), want)
            assert mx < 2e-6 and fro < 2e-6, (mx, fro)
    grp.close()


def test_group_equals_one_call_at_a_time(ctx, torch_cuda):
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(33)
    items, host = _sweep_items(torch, t1m, rng, 4, [16, 32, 64], [2, 4])
    grp = t1m.Group(items, ctx=ctx, graph=True)
    grp.launch()
    grouped = [(r1.clone(), out.clone()) for _, _, _, r1, out, _ in host]
    for (alpha, a, la, b, lb, beta, c, lc, _dep) in items:
        t1m.contract_scaled(alpha, a, la, b, lb, beta, c, lc, ctx=ctx)
    torch.cuda.synchronize()
    # Both may pick different kernels per item (the group's skinny plain tile
    # vs the per-call choice), so both are held to the FP64 oracle; the plain
    # form's sequential FP32 error grows like u*sqrt(2K).
    for (g_r1, g_out), (X1, X2, X3, r1, out, _) in zip(grouped, host):
        R = np.einsum("xay,asb->xsyb", X1.astype(np.complex128), X2.astype(np.complex128))
        ref = np.einsum("xsyb,ytb->xst", R, X3.astype(np.complex128))
        k2 = X3.shape[0] * X3.shape[2]
        tol = max(2e-6, 4 * 2.0 ** -24 * np.sqrt(2.0 * k2))
        for got in (g_out, out):
            mx, _ = no.rel_errors(got.cpu().numpy(), ref)
            assert mx < tol, (mx, tol)
        for got in (g_r1, r1):
            mx, _ = no.rel_errors(got.cpu().numpy(), R)
            assert mx < 2e-6, mx
    grp.close()


def test_group_rejects_forward_dependency_and_host_data(ctx, torch_cuda):
    import t1m_gb300 as t1m
    A = np.ones((2, 3), np.complex64)
    B = np.ones((3, 2), np.complex64)
    Cm = np.zeros((2, 2), np.complex64)
    v = t1m.tensor.from_array
    with pytest.raises(t1m.T1MError):
        t1m.Group([(1.0, v(A), "ab", v(B), "bc", 0.0, v(Cm), "ac", -1)], ctx=ctx)
    torch = torch_cuda
    g = [torch.from_numpy(x).cuda() for x in (A, B, Cm)]
    w = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    with pytest.raises(t1m.T1MError):
        t1m.Group([(1.0, w(g[0]), "ab", w(g[1]), "bc", 0.0, w(g[2]), "ac", 1)], ctx=ctx)


@pytest.mark.parametrize("one_launch", [False, True], ids=["per-family", "one-launch"])
def test_group_split_k_long_contractions(ctx, torch_cuda, one_launch):
    """Items whose K exceeds the per-tile cap are split across CTAs (partials in
    the group's workspace): a wide item, a skinny item, their dependents,
    complex alpha and a nonzero beta applied by the reduction.  As one
    persistent launch the reduction runs in the kernel (the split that
    finishes last sums the partials in FP64); per family, one FP64 reduction
    launch per dependency level."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(34)
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    X = _rand(rng, (96, 3000), np.complex64, 0.1)
    Y = _rand(rng, (3000, 160), np.complex64, 0.1)
    P = _rand(rng, (200, 5000), np.complex64, 0.1)
    Q = _rand(rng, (5000, 3), np.complex64, 0.1)
    Z = _rand(rng, (160, 64), np.complex64, 0.1)
    W = _rand(rng, (3, 40), np.complex64, 0.1)
    C0 = _rand(rng, (200, 3), np.complex64, 1.0)
    g = {k: torch.from_numpy(a.copy()).cuda() for k, a in
         dict(X=X, Y=Y, P=P, Q=Q, Z=Z, W=W, C0=C0).items()}
    r1 = torch.zeros((96, 160), dtype=torch.complex64, device="cuda")
    r2 = g["C0"].clone()
    o1 = torch.zeros((96, 64), dtype=torch.complex64, device="cuda")
    o2 = torch.zeros((200, 40), dtype=torch.complex64, device="cuda")
    al = 0.5 - 0.25j
    items = [(1.0, v(g["X"]), "xa", v(g["Y"]), "ay", 0.0, v(r1), "xy", -1),
             (al, v(g["P"]), "xa", v(g["Q"]), "at", 0.5, v(r2), "xt", -1),
             (1.0, v(r1), "xy", v(g["Z"]), "yq", 0.0, v(o1), "xq", 0),
             (1.0, v(r2), "xt", v(g["W"]), "tz", 0.0, v(o2), "xz", 1)]
    grp = t1m.Group(items, ctx=ctx, graph=True,
                    options=t1m.GROUP_ONE_LAUNCH if one_launch else 0)
    rep = grp.launch()
    if not one_launch:
        # Two levels, each with main launches and one reduction.
        assert rep.kernels >= 3
    else:
        assert rep.kernels == 1
    d = lambda z: z.astype(np.complex128)  # noqa: E731
    R1 = d(X) @ d(Y)
    R2 = al * (d(P) @ d(Q)) + 0.5 * d(C0)
    for got, want, tol in ((r1, R1, 2e-6), (r2, R2, 4e-6), (o1, R1 @ d(Z), 2e-6),
                           (o2, R2 @ d(W), 4e-6)):
        mx, fro = no.rel_errors(got.cpu().numpy(), want)
        assert mx < tol and fro < tol, (mx, fro, tol)
    grp.close()


@pytest.mark.parametrize("dt", [np.complex64, np.float64])
def test_group_skinny_outputs(ctx, torch_cuda, dt):
    """Grouped items with at most 16 output columns run on the skinny kernel:
    A with unit K stride (one warp per row) and with unit M stride (one
    thread per row), N = 3 and N = 13 (the 4- and 16-column instances), a
    long K that is split, alpha and beta applied through the reduction."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(35)

    def r(shape):
        x = rng.uniform(-1, 1, shape)
        if np.dtype(dt).kind == "c":
            x = x + 1j * rng.uniform(-1, 1, shape)
        return x.astype(dt)

    # C-ordered arrays, handed over as col-major views with reversed extents
    # and labels: the last label of each string is the unit-stride mode.
    cases = [("ak", "kn", "an", dict(a=300, k=5000, n=3)),    # K unit stride
             ("ka", "kn", "an", dict(a=700, k=2100, n=13)),   # M unit stride
             ("ak", "kn", "an", dict(a=37, k=64, n=13))]      # short K, ragged rows
    items, checks = [], []
    v = lambda z: t1m.tensor(list(z.shape)[::-1], z, t1m.col_major)  # noqa: E731
    alpha = 0.5 - 0.25j if np.dtype(dt).kind == "c" else 0.5
    for la, lb, lc, ext in cases:
        A, B = r([ext[c] for c in la]), r([ext[c] for c in lb])
        C0 = r([ext[c] for c in lc])
        ga, gb, gc = (torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (A, B, C0))
        items.append((alpha, v(ga), la[::-1], v(gb), lb[::-1], 0.25, v(gc), lc[::-1], -1))
        ref = alpha * np.einsum(f"{la},{lb}->{lc}", A.astype(np.complex128),
                                B.astype(np.complex128)) + 0.25 * C0.astype(np.complex128)
        checks.append((gc, ref, (ga, gb)))
    grp = t1m.Group(items, ctx=ctx, graph=True)
    grp.launch()
    tol = 2e-6 if np.dtype(dt) == np.complex64 else 1e-12
    for gc, ref, _ in checks:
        mx, fro = no.rel_errors(gc.cpu().numpy().astype(np.complex128), ref)
        assert mx < tol and fro < tol, (mx, fro)
    grp.close()


def _width_batch(torch, t1m, rng):
    """complex64 items of every width class: N from 1 to 300 (ragged against
    each tile width), TMA and gathered operands (row-major tensors, and a
    permuted A), short and long K (split, reduced in the kernel), complex
    alpha, nonzero beta, accumulation, conjugation, and items that read the
    C of earlier items."""
    d = lambda z: z.astype(np.complex128)  # noqa: E731
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    items, checks, keep = [], [], []
    specs = [  # (M, N, K, alpha, beta, flags)
        (96, 1, 700, 1.0, 0.0, 0),
        (200, 3, 5000, 0.5 - 0.25j, 0.5, 0),
        (130, 13, 64, 1.0, 0.0, t1m.FLAG_CONJ_A),
        (64, 16, 2100, 1.0, 0.25, t1m.FLAG_CONJ_B),
        (77, 17, 48, 1j, 0.0, 0),
        (150, 40, 3000, 1.0, 0.0, t1m.FLAG_ACCUMULATE),
        (64, 64, 96, 1.0, 0.0, t1m.FLAG_CONJ_A | t1m.FLAG_CONJ_B),
        (100, 100, 1030, 0.75, -0.5j, 0),
        (257, 130, 80, 1.0, 0.0, 0),
        (40, 300, 1500, 1.0, 0.0, 0),
    ]
    for (M, N, K, al, be, fl) in specs:
        A = _rand(rng, (M, K), np.complex64, 0.2)
        B = _rand(rng, (K, N), np.complex64, 0.2)
        C0 = _rand(rng, (M, N), np.complex64, 1.0)
        ga, gb, gc = (torch.from_numpy(x.copy()).cuda() for x in (A, B, C0))
        a_ = d(A).conj() if fl & t1m.FLAG_CONJ_A else d(A)
        b_ = d(B).conj() if fl & t1m.FLAG_CONJ_B else d(B)
        prod = al * (a_ @ b_)
        if fl & t1m.FLAG_ACCUMULATE:
            ref = d(C0) + prod
        else:
            ref = prod + be * d(C0)
        items.append((al, v(ga), "mk", v(gb), "kn", be, v(gc), "mn", -1, fl))
        checks.append((gc, ref))
        keep += [ga, gb]
    # A permuted (gathered) A: labels "km" over a row-major (K, M) array.
    M, N, K = 120, 24, 900
    At = _rand(rng, (K, M), np.complex64, 0.2)
    B = _rand(rng, (K, N), np.complex64, 0.2)
    ga, gb = (torch.from_numpy(x.copy()).cuda() for x in (At, B))
    gc = torch.zeros((M, N), dtype=torch.complex64, device="cuda")
    items.append((1.0, v(ga), "km", v(gb), "kn", 0.0, v(gc), "mn", -1))
    checks.append((gc, d(At).T @ d(B)))
    keep += [ga, gb]
    # Dependents: read the C of items 1 (N = 3, split) and 7 (N = 100).
    for dep, (Md, Nd) in ((1, (200, 3)), (7, (100, 100))):
        Q = _rand(rng, (Nd, 5), np.complex64, 0.2)
        gq = torch.from_numpy(Q.copy()).cuda()
        go = torch.zeros((Md, 5), dtype=torch.complex64, device="cuda")
        items.append((1.0, items[dep][6], "mn", v(gq), "nq", 0.0, v(go), "mq", dep))
        checks.append((go, checks[dep][1] @ d(Q)))
        keep.append(gq)
    return items, checks, keep


@pytest.mark.parametrize("width", [0, 16, 32, 64, 128], ids=lambda w: f"w{w}" if w else "auto")
def test_one_launch_tile_widths(ctx, torch_cuda, width):
    """A complex64 batch under GROUP_ONE_LAUNCH is ONE persistent launch
    (report: one kernel), each item with its own tile (chosen per item: SIMT
    tiles for N <= 8, else a tensor-core width; or a width forced for every
    item wider than 8 columns), long K split and reduced in the kernel, dependencies resolved in
    the kernel; every output against FP64, on two launches in a row (the
    in-kernel split counters reset themselves)."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(36)
    items, checks, keep = _width_batch(torch, t1m, rng)
    inits = [c.clone() for c, _ in checks]
    grp = t1m.Group(items, ctx=ctx, graph=True, options=t1m.GROUP_ONE_LAUNCH | width)
    for rnd in range(2):
        for (c, _), c0 in zip(checks, inits):
            c.copy_(c0)
        torch.cuda.synchronize()
        rep = grp.launch()
        assert rep.kernels == 1
        for i, (c, ref) in enumerate(checks):
            mx, fro = no.rel_errors(c.cpu().numpy(), ref)
            assert mx < 2e-6 and fro < 2e-6, (rnd, i, mx, fro)
    grp.close()


def test_one_launch_width_autotune(ctx, torch_cuda, tmp_path, monkeypatch):
    """The autotuner picks a tile per shape class (a tensor-core width, or a
    SIMT tile for outputs of at most 8 columns; cached in the tune file) and
    the batch stays one launch with results within FP32 rounding of FP64."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    monkeypatch.setenv("T1M_TUNE_CACHE", str(tmp_path / "tune.txt"))
    rng = np.random.default_rng(37)
    items, checks, keep = _width_batch(torch, t1m, rng)
    grp = t1m.Group(items, ctx=ctx, graph=True, autotune=True, options=t1m.GROUP_ONE_LAUNCH)
    rep = grp.launch()
    assert rep.kernels == 1
    for i, (c, ref) in enumerate(checks):
        mx, fro = no.rel_errors(c.cpu().numpy(), ref)
        assert mx < 2e-6 and fro < 2e-6, (i, mx, fro)
    grp.close()
    lines = (tmp_path / "tune.txt").read_text().splitlines()
    # Tile choices: 1 = a SIMT tile (outputs of at most 8 columns), else the
    # tensor-core tile width.
    widths = [int(ln.split()[1]) for ln in lines[1:] if ln.startswith("w")]
    assert widths and set(widths) <= {1, 16, 32, 64, 128}
