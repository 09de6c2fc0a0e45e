"""Parity at the configured sizes (gpu): every kernel the workloads run,
checked against FP64.

* Differentiation form: abcd,ebfd->aecf with all extents 32, dA and dB from
  the adjoint, against gradients assembled from the reference algorithm's
  own contract calls on conj(B) and conj(A) (the oracle port, in complex128)
  and against complex128 central differences; both operand paths: the
  default (A packed densely, B split into panels) and the per-16-row block
  TMA modes of the adjoint layouts (optional workspaces off).
* Precision form at M = N = K = 4096: 3xTF32 and the automatic method on both
  input sets; the complex128 companion on DMMA and on the plain FP64 kernel.
* Batching form: the full batch of 1024 sweep updates as one grouped launch
  under a CUDA graph, every item checked on sampled outputs.
* The automatic method's precision rule: long contractions are split along K
  so that every FP32 partial stays within 1e-6, partials summed in FP64.
"""
import os

import numpy as np
import pytest

from oracle import libs
from oracle import numpy_oracle as no

pytestmark = pytest.mark.gpu

TOL = 1e-6  # normwise max relative error against FP64 (the spec bar)


def _rows(torch, x):
    import t1m_gb300 as t1m
    return t1m.tensor(list(x.shape), x, t1m.row_major)


# ------------------------------------------------------- differentiation ---
E5 = 32
L5 = ("abcd", "ebfd", "aecf")


@pytest.fixture(scope="module")
def cfg5(torch_cuda):
    """Inputs of the differentiation form and the reference-assembled
    gradients: dA = contract(dC, conj(B)), dB = contract(conj(A), dC), each one
    call of the reference algorithm (oracle port) in complex128 on the same
    (upcast) complex64 inputs, all host cores."""
    torch = torch_cuda
    g = torch.Generator(device="cuda")
    g.manual_seed(9)

    def mk():
        return torch.complex(torch.rand((E5,) * 4, device="cuda", generator=g) * 2 - 1,
                             torch.rand((E5,) * 4, device="cuda", generator=g) * 2 - 1)

    A, B, G = mk(), mk(), mk()
    dims = [E5] * 4
    rm = no.row_major_strides(dims)
    la, lb, lc = L5
    threads = os.cpu_count() or 1

    def port(x, lx, y, ly, lz):
        out = np.zeros(E5 ** 4, np.complex128)
        libs.port_contract(np.ascontiguousarray(x.reshape(-1)), dims, rm, lx,
                           np.ascontiguousarray(y.reshape(-1)), dims, rm, ly, out, dims, rm, lz,
                           nthreads=threads)
        return out

    a64, b64, g64 = (z.cpu().numpy().astype(np.complex128) for z in (A, B, G))
    dA_ref = port(g64, lc, np.conj(b64), lb, la)
    dB_ref = port(np.conj(a64), la, g64, lc, lb)
    return A, B, G, dA_ref, dB_ref


# Fetch paths of the two adjoint products with the optional workspaces off
# (t1m_set_workspace_limit(0)): the per-16-row block TMA modes.
BLOCK_PATHS = {"dA": ("KM16", "KN16"), "dB": ("MK16K", "KN16")}


@pytest.mark.parametrize("workspace", ["default", "none"])
@pytest.mark.parametrize("method", ["auto", "tc_3xtf32", "tc_bf16x6"])
def test_config5_adjoint_full_size(ctx, torch_cuda, cfg5, method, workspace):
    import t1m_gb300 as t1m
    torch = torch_cuda
    A, B, G, dA_ref, dB_ref = cfg5
    la, lb, lc = L5
    ctx.set_method(method)
    ctx.set_workspace_limit(0 if workspace == "none" else -1)
    try:
        for name, ref in (("dA", dA_ref), ("dB", dB_ref)):
            out = torch.empty_like(A if name == "dA" else B)
            args = (_rows(torch, out), None) if name == "dA" else (None, _rows(torch, out))
            rep = t1m.contract_vjp(_rows(torch, G), lc, _rows(torch, A), la, _rows(torch, B), lb,
                                   *args, ctx=ctx)
            torch.cuda.synchronize()
            got = out.cpu().numpy().reshape(-1).astype(np.complex128)
            mx, fro = no.rel_errors(got, ref)
            assert mx <= TOL and fro <= TOL, (name, method, workspace, mx, fro)
            f = rep.fetch
            assert f is not None, rep.path
            if workspace == "default":
                # Dense pack of the gathered A, B split once into panels, both
                # loaded by TMA on the one-tile kernel.
                assert f["a_packed"] and f["b"] == "panels" and not f["persistent"], f
            elif method == "tc_bf16x6":
                # The bf16 forms run only on the one-tile kernel: block-mode
                # operands are gathered there.
                assert not f["persistent"] and (f["a"], f["b"]) == ("gather", "gather"), f
            else:
                assert f["persistent"] and (f["a"], f["b"]) == BLOCK_PATHS[name], f
                assert rep.method == t1m.method.tc_3xtf32
    finally:
        ctx.set_workspace_limit(-1)
        ctx.set_method("auto")


def test_config5_adjoint_finite_differences(ctx, torch_cuda, cfg5):
    """Directional central differences (step 1e-6) of the complex128 loss
    L = Re sum conj(dC) * (A*B) against the complex64 adjoint's gradients.

    Along the FP64 gradient itself the derivative is |grad|^2 (no
    cancellation), so it is held to 1e-6 relative.  Along a random direction
    V the derivative is a sum of a million terms of either sign; there the
    normwise bound |<dA - grad, V>| <= 1e-6 |grad| |V| applies."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    A, B, G, _, _ = cfg5
    la, lb, lc = L5
    dA, dB = torch.empty_like(A), torch.empty_like(B)
    t1m.contract_vjp(_rows(torch, G), lc, _rows(torch, A), la, _rows(torch, B), lb,
                     _rows(torch, dA), _rows(torch, dB), ctx=ctx)
    a, b, gc = (z.to(torch.complex128) for z in (A, B, G))
    grad_a = torch.einsum("aecf,ebfd->abcd", gc, b.conj())
    grad_b = torch.einsum("abcd,aecf->ebfd", a.conj(), gc)

    def loss(x, y):
        return torch.sum(torch.conj(gc) * torch.einsum("abcd,ebfd->aecf", x, y)).real.item()

    gen = torch.Generator(device="cuda")
    gen.manual_seed(13)

    def rand_dir():
        return torch.complex(
            torch.rand(a.shape, device="cuda", generator=gen, dtype=torch.float64) * 2 - 1,
            torch.rand(a.shape, device="cuda", generator=gen, dtype=torch.float64) * 2 - 1)

    h = 1e-6
    for va, vb, along in ((grad_a, grad_b, True), (rand_dir(), rand_dir(), False)):
        fd_a = (loss(a + h * va, b) - loss(a - h * va, b)) / (2 * h)
        fd_b = (loss(a, b + h * vb) - loss(a, b - h * vb)) / (2 * h)
        an_a = torch.sum(torch.conj(dA.to(torch.complex128)) * va).real.item()
        an_b = torch.sum(torch.conj(dB.to(torch.complex128)) * vb).real.item()
        if along:
            bound_a, bound_b = TOL * abs(an_a), TOL * abs(an_b)
        else:
            bound_a = TOL * (torch.linalg.vector_norm(grad_a) * torch.linalg.vector_norm(va)).item()
            bound_b = TOL * (torch.linalg.vector_norm(grad_b) * torch.linalg.vector_norm(vb)).item()
        assert abs(fd_a - an_a) <= bound_a, (along, fd_a, an_a)
        assert abs(fd_b - an_b) <= bound_b, (along, fd_b, an_b)


# ------------------------------------------------------------ precision ---
def _config3_inputs(torch, inputs, dtype, seed=21):
    n = 4096 * 4096
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    rdt = torch.float32 if dtype == torch.complex64 else torch.float64
    if inputs == "uniform":
        def mk():
            return torch.complex(torch.rand(n, device="cuda", generator=g, dtype=rdt) * 2 - 1,
                                 torch.rand(n, device="cuda", generator=g, dtype=rdt) * 2 - 1)
    else:
        def mk():
            mag = torch.pow(10.0, torch.rand(n, device="cuda", generator=g, dtype=rdt) * 6 - 3)
            ph = torch.rand(n, device="cuda", generator=g, dtype=rdt) * 2 * np.pi
            return torch.polar(mag, ph)
    return mk(), mk()


def _config3_check(ctx, torch, ga, gb, methods, tol, samples=512):
    import t1m_gb300 as t1m
    dims = [64] * 4
    fa, fb = ga.cpu().numpy(), gb.cpu().numpy()
    st = no.col_major_strides(dims)
    scat = no.matricize("ijkl", "klmn", "ijmn", dims, dims, dims, st, st, st)
    rng = np.random.default_rng(3)
    rows, cols = rng.integers(0, 4096, samples), rng.integers(0, 4096, samples)
    ref = no.sampled_entries(fa, fb, scat, rows, cols)
    off = scat[4][rows] + scat[5][cols]
    out = {}
    for m in methods:
        ctx.set_method(m)
        gc = torch.zeros(4096 * 4096, dtype=ga.dtype, device="cuda")
        rep = t1m.contract_scaled(1.0, t1m.tensor(dims, ga), "ijkl", t1m.tensor(dims, gb),
                                  "klmn", 0.0, t1m.tensor(dims, gc), "ijmn", ctx=ctx)
        torch.cuda.synchronize()
        got = gc.cpu().numpy()[off].astype(np.complex128)
        mx, fro = no.rel_errors(got, ref)
        assert mx <= tol and fro <= tol, (m, mx, fro)
        out[m] = rep
    ctx.set_method("auto")
    return out


@pytest.mark.slow
@pytest.mark.parametrize("inputs", ["uniform", "logmag"])
def test_config3_3xtf32_full_size(ctx, torch_cuda, inputs):
    """complex64 ijkl,klmn->ijmn at 4096^3, both input sets: 3xTF32 and the
    automatic method (BF16x6), on CTA pairs (the automatic tile form) and on
    one tile per CTA (3xTF32 with B panels), within 1e-6 of sampled FP64."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    ga, gb = _config3_inputs(torch, inputs, torch.complex64)
    reps = _config3_check(ctx, torch, ga, gb, ["tc_3xtf32", "auto"], TOL)
    assert reps["tc_3xtf32"].method == t1m.method.tc_3xtf32
    assert reps["tc_3xtf32"].fetch["pair"] and reps["auto"].fetch["pair"]
    assert reps["auto"].method == t1m.method.tc_bf16x6
    ctx.set_tile_form("one")
    try:
        reps = _config3_check(ctx, torch, ga, gb, ["tc_3xtf32"], TOL)
    finally:
        ctx.set_tile_form("auto")
    assert reps["tc_3xtf32"].fetch["b"] == "panels" and not reps["tc_3xtf32"].fetch["pair"]


@pytest.mark.slow
@pytest.mark.parametrize("inputs", ["uniform", "logmag"])
def test_config3_complex128_full_size(ctx, torch_cuda, inputs):
    """The complex128 companion at 4096^3: FP64 tensor cores (DMMA) and the
    automatic method (plain FP64), within 1e-12 of sampled FP64 dot products."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    ga, gb = _config3_inputs(torch, inputs, torch.complex128)
    reps = _config3_check(ctx, torch, ga, gb, ["dmma", "auto"], 1e-12, samples=256)
    assert reps["dmma"].method == t1m.method.dmma
    assert reps["auto"].method == t1m.method.plain


# -------------------------------------------------------------- batching ---
def _sweep_batch(torch, n_items, seed=2024):
    """The batching form's items, drawn as the benchmark draws them: bonds x,
    y, a, b from {16, ..., 256}, physical s, t from {2, 4}, components
    N(0, 1/sqrt(bond))."""
    import t1m_gb300 as t1m
    rng = np.random.default_rng(seed)
    bonds = np.arange(16, 257, 16)
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    items, keep = [], []
    for _ in range(n_items):
        x, y, a, b = (int(w) for w in rng.choice(bonds, 4))
        s, t = (int(w) for w in rng.choice([2, 4], 2))

        def mk(shape, bond):
            sc = 1.0 / np.sqrt(np.sqrt(bond))
            return torch.complex(torch.randn(shape, device="cuda", generator=g) * sc,
                                 torch.randn(shape, device="cuda", generator=g) * sc)

        X1, X2, X3 = mk((x, a, y), a), mk((a, s, b), a), mk((y, t, b), b)
        R = torch.full((x, s, y, b), float("nan"), dtype=torch.complex64, device="cuda")
        O = torch.full((x, s, t), float("nan"), dtype=torch.complex64, device="cuda")
        i1 = len(items)
        items.append((1.0, v(X1), "xay", v(X2), "asb", 0.0, v(R), "xsyb", -1))
        items.append((1.0, v(R), "xsyb", v(X3), "ytb", 0.0, v(O), "xst", i1))
        keep.append((X1, X2, X3, R, O))
    return items, keep


@pytest.mark.slow
@pytest.mark.parametrize("one_launch", [False, True], ids=["per-family", "one-launch"])
def test_config4_full_batch_grouped_graph(ctx, torch_cuda, one_launch):
    """All 1024 updates (2048 contractions) under a CUDA graph with the
    autotuner, as family launches per level and as ONE persistent launch; every item's outputs checked against FP64 on
    sampled rows: R[x, s, :, :] (all y, b of one x, s) and O[x, :, :] for
    four x (all s, t; O rows hold only 2-4 entries, too few to normalise
    the error by on their own)."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    items, keep = _sweep_batch(torch, 1024)
    grp = t1m.Group(items, ctx=ctx, graph=True, autotune=True,
                    options=t1m.GROUP_ONE_LAUNCH if one_launch else 0)
    try:
        grp.launch(timed=False)
        rep = grp.launch()  # a graph replay over the same outputs
        torch.cuda.synchronize()
    finally:
        grp.close()
    # One persistent launch, or per level the family launches and reduction.
    assert rep.kernels == 1 if one_launch else rep.kernels >= 2
    rng = np.random.default_rng(17)
    worst = (0.0, None)
    c128 = torch.complex128
    for i, (X1, X2, X3, R, O) in enumerate(keep):
        x, s = int(rng.integers(X1.shape[0])), int(rng.integers(X2.shape[1]))
        # R[x, s, :, :] = X1[x]^T X2[:, s, :]
        r_ref = X1[x].to(c128).t() @ X2[:, s, :].to(c128)
        xs = torch.from_numpy(rng.integers(0, X1.shape[0], 4)).cuda()
        o_ref = torch.einsum("xsyb,ytb->xst",
                             torch.einsum("xay,asb->xsyb", X1[xs].to(c128), X2.to(c128)),
                             X3.to(c128))
        for name, got, ref in (("R", R[x, s], r_ref), ("O", O[xs], o_ref)):
            e = ((got.to(c128) - ref).abs().max() / ref.abs().max()).item()
            assert e == e, (i, name, "unwritten output (NaN)")
            if e > worst[0]:
                worst = (e, (i, name, tuple(X1.shape), tuple(X2.shape), tuple(X3.shape)))
    assert worst[0] <= TOL, worst


# -------------------------------------------------------- precision rule ---
@pytest.mark.parametrize("case", [
    # complex64 on the tensor cores: K = 16384 > 4096 per FP32 partial.
    (np.complex64, 1024, 1024, 16384, 4),
    # float32 on the tensor cores: K = 32768 > 8192.
    (np.float32, 1024, 1024, 32768, 4),
    # complex64 on the plain kernel (M*N*K < 2^18): K = 32768 > 128.
    (np.complex64, 2, 2, 32768, 256),
], ids=["c64-tc", "f32-tc", "c64-plain"])
def test_auto_splits_long_k_for_1e6(ctx, torch_cuda, case):
    """T1M_METHOD_AUTO keeps every FP32-accumulated partial within its K
    limit (split-K, FP64 reduction and epilogue) and meets 1e-6 against
    sampled FP64."""
    torch = torch_cuda
    import t1m_gb300 as t1m
    dt, M, N, K, min_splits = case
    rng = np.random.default_rng(4)

    def r(n):
        x = rng.uniform(-1, 1, n)
        if np.dtype(dt).kind == "c":
            x = x + 1j * rng.uniform(-1, 1, n)
        return x.astype(dt)

    fa, fb = r(M * K), r(K * N)
    ga, gb = torch.from_numpy(fa).cuda(), torch.from_numpy(fb).cuda()
    gc = torch.zeros(M * N, dtype=ga.dtype, device="cuda")
    ctx.set_method("auto")
    rep = t1m.contract_scaled(1.0, t1m.tensor([M, K], ga), "mk", t1m.tensor([K, N], gb), "kn",
                              0.0, t1m.tensor([M, N], gc), "mn", ctx=ctx)
    torch.cuda.synchronize()
    assert rep.split_k >= min_splits, rep.split_k
    dims = ([M, K], [K, N], [M, N])
    scat = no.matricize("mk", "kn", "mn", *dims, *(no.col_major_strides(d) for d in dims))
    rows = rng.integers(0, M, 256)
    cols = rng.integers(0, N, 256)
    ref = no.sampled_entries(fa, fb, scat, rows, cols)
    got = gc.cpu().numpy()[scat[4][rows] + scat[5][cols]].astype(np.complex128)
    mx, fro = no.rel_errors(got, ref)
    assert mx <= TOL and fro <= TOL, (mx, fro, rep.split_k)
