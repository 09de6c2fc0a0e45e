"""Batch (Hadamard) labels — a label of A, B and C alike — against the FP64
oracle (gpu).  The reference leaves such labels undefined (t1m.h:100-135); here
the contraction is one independent product per batch index."""
import numpy as np
import pytest

from oracle import numpy_oracle as no

pytestmark = pytest.mark.gpu

CASES = [
    ("bij", "bjk", "bik", dict(b=5, i=70, j=33, k=40)),      # batched matrix product
    ("abc", "acd", "abd", dict(a=3, b=20, c=64, d=16)),      # batch first in every tensor
    ("iab", "bca", "cai", dict(a=6, b=24, c=18, i=9)),       # batch label a, permuted positions
    ("ij", "ij", "ij", dict(i=6, j=7)),                      # pure Hadamard (M = N = K = 1)
    ("ab", "ac", "abc", dict(a=4, b=10, c=12)),              # batch with an empty K (outer)
]

TOL = {np.dtype(np.complex64): 2e-5, np.dtype(np.float64): 1e-12,
       np.dtype(np.complex128): 1e-12}


def _rand(rng, shape, dt):
    x = rng.uniform(-1, 1, shape)
    if np.dtype(dt).kind == "c":
        x = x + 1j * rng.uniform(-1, 1, shape)
    return x.astype(dt)


def _methods(dt):
    if np.dtype(dt) == np.complex64:
        return ["auto", "plain", "tc_3xtf32", "tc_bf16x6"]
    return ["auto", "plain", "dmma"]


@pytest.mark.parametrize("dt", [np.complex64, np.float64, np.complex128])
@pytest.mark.parametrize("layout", ["col", "row"])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_batch_labels_host_buffers(ctx, case, layout, dt):
    import t1m_gb300 as t1m
    la, lb, lc, ext = CASES[case]
    da, db, dc = ([ext[ch] for ch in s] for s in (la, lb, lc))
    order = "F" if layout == "col" else "C"
    L = t1m.col_major if layout == "col" else t1m.row_major
    rng = np.random.default_rng(40 + case)
    A, B, C0 = _rand(rng, da, dt), _rand(rng, db, dt), _rand(rng, dc, dt)
    alpha = (1 + 0.5j) if np.dtype(dt).kind == "c" else 1.5
    beta = 0.25
    ref = no.contract_fp64(A, la, B, lb, C0, lc, alpha=alpha, beta=beta)
    for m in _methods(dt):
        ctx.set_method(m)
        fc = C0.flatten(order=order)
        try:
            rep = t1m.contract_scaled(alpha, t1m.tensor(da, A.flatten(order=order), L), la,
                                      t1m.tensor(db, B.flatten(order=order), L), lb, beta,
                                      t1m.tensor(dc, fc, L), lc, ctx=ctx)
        finally:
            ctx.set_method("auto")
        got = fc.reshape(dc, order=order)
        mx, fro = no.rel_errors(got, ref)
        assert mx < TOL[np.dtype(dt)] and fro < TOL[np.dtype(dt)], (m, mx, fro)
        batch = int(np.prod([ext[ch] for ch in set(la) & set(lb) & set(lc)]))
        assert rep.kernels >= batch


def test_batch_labels_device_buffers_reference_semantics(ctx, torch_cuda):
    """Device tensors, C += A*B (the reference's contract semantics)."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(50)
    A = _rand(rng, (4, 48, 40), np.complex64)     # b i j (row-major)
    B = _rand(rng, (4, 40, 56), np.complex64)     # b j k
    C0 = _rand(rng, (4, 48, 56), np.complex64)    # b i k
    ga, gb, gc = (torch.from_numpy(x.copy()).cuda() for x in (A, B, C0))
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    t1m.contract(v(ga), "bij", v(gb), "bjk", v(gc), "bik", ctx=ctx)
    torch.cuda.synchronize()
    ref = C0.astype(np.complex128) + np.einsum("bij,bjk->bik", A.astype(np.complex128),
                                               B.astype(np.complex128))
    mx, fro = no.rel_errors(gc.cpu().numpy(), ref)
    assert mx < 2e-6 and fro < 2e-6, (mx, fro)


def test_batch_labels_vjp(ctx, torch_cuda):
    """The adjoint with a batch label: dA = dC * conj(B), dB = conj(A) * dC per
    batch index."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(51)
    A = _rand(rng, (3, 20, 16), np.complex128)    # b i j
    B = _rand(rng, (3, 16, 24), np.complex128)    # b j k
    G = _rand(rng, (3, 20, 24), np.complex128)    # b i k
    ga, gb, gg = (torch.from_numpy(x.copy()).cuda() for x in (A, B, G))
    da, db = torch.zeros_like(ga), torch.zeros_like(gb)
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    t1m.contract_vjp(v(gg), "bik", v(ga), "bij", v(gb), "bjk", v(da), v(db), ctx=ctx)
    torch.cuda.synchronize()
    rA = np.einsum("bik,bjk->bij", G, np.conj(B))
    rB = np.einsum("bij,bik->bjk", np.conj(A), G)
    assert no.rel_errors(da.cpu().numpy(), rA)[0] < 1e-12
    assert no.rel_errors(db.cpu().numpy(), rB)[0] < 1e-12


def test_batch_labels_rejected_in_groups(ctx, torch_cuda):
    import t1m_gb300 as t1m
    torch = torch_cuda
    g = [torch.zeros(s, dtype=torch.complex64, device="cuda") for s in ((2, 3, 4), (2, 4, 5),
                                                                         (2, 3, 5))]
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    with pytest.raises(t1m.T1MError):
        t1m.Group([(1.0, v(g[0]), "bij", v(g[1]), "bjk", 0.0, v(g[2]), "bik", -1)], ctx=ctx)
