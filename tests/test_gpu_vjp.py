"""Adjoint (t1m_contract_vjp) and the recomputing contraction chain (gpu).

Checked against
  * gradients assembled from the reference algorithm's own contract calls on
    conj(B) and conj(A) (the oracle port, bit-identical to the reference),
  * complex128 central finite differences (step 1e-6) of the real loss
    L = Re <dC, A*B> along random directions,
  * torch.autograd.gradcheck of the autograd wrapper (complex128).
"""
import numpy as np
import pytest

from oracle import libs
from oracle import numpy_oracle as no

pytestmark = pytest.mark.gpu


def _rand(rng, shape, dt):
    x = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
    return x.astype(dt)


def _dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


CASES = [("abcd", "ebfd", "aecf", dict(a=4, b=5, c=3, d=6, e=4, f=5)),
         ("abc", "bd", "acd", dict(a=7, b=9, c=5, d=6)),
         ("xay", "asb", "xsyb", dict(x=6, a=8, y=5, s=2, b=7))]


@pytest.mark.parametrize("method", ["plain", "tc_3xtf32"])
@pytest.mark.parametrize("case", CASES, ids=lambda c: ",".join(c[:3]))
def test_vjp_matches_reference_assembled_gradients(ctx, torch_cuda, case, method):
    """dA = contract(dC, conj(B)) and dB = contract(conj(A), dC), each computed
    by the reference algorithm (port) in complex64, vs the GPU adjoint."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    la, lb, lc, ext = case
    rng = np.random.default_rng(8)
    A = _rand(rng, [ext[c] for c in la], np.complex64)
    B = _rand(rng, [ext[c] for c in lb], np.complex64)
    G = _rand(rng, [ext[c] for c in lc], np.complex64)
    # Reference-assembled gradients (column-major buffers through the port).
    cm = no.col_major_strides

    def port(x, lx, y, ly, lz):
        dz = [ext[c] for c in lz]
        out = np.zeros(int(np.prod(dz)), np.complex64)
        fx, fy = x.reshape(-1, order="F").copy(), y.reshape(-1, order="F").copy()
        libs.port_contract(fx, list(x.shape), cm(x.shape), lx, fy, list(y.shape), cm(y.shape),
                           ly, out, dz, cm(dz), lz)
        return out.reshape(dz, order="F")

    dA_ref = port(G, lc, np.conj(B), lb, la)
    dB_ref = port(np.conj(A), la, G, lc, lb)
    ctx.set_method(method)
    ga, gb, gg = _dev(torch, A), _dev(torch, B), _dev(torch, G)
    da, db = torch.empty_like(ga), torch.empty_like(gb)
    v = lambda x: t1m.tensor(list(x.shape), x, t1m.row_major)  # noqa: E731
    rep = t1m.contract_vjp(v(gg), lc, v(ga), la, v(gb), lb, v(da), v(db), ctx=ctx)
    ctx.set_method("auto")
    assert rep.kernels >= 2
    for got, ref in ((da, dA_ref), (db, dB_ref)):
        g = got.cpu().numpy()
        assert np.abs(g - ref).max() / np.abs(ref).max() < 2e-5


@pytest.mark.parametrize("case", CASES, ids=lambda c: ",".join(c[:3]))
def test_vjp_finite_differences_complex128(ctx, torch_cuda, case):
    """Directional central differences of L = Re sum conj(G) * (A*B), step 1e-6."""
    import t1m_gb300 as t1m
    torch = torch_cuda
    la, lb, lc, ext = case
    rng = np.random.default_rng(9)
    A = _rand(rng, [ext[c] for c in la], np.complex128)
    B = _rand(rng, [ext[c] for c in lb], np.complex128)
    G = _rand(rng, [ext[c] for c in lc], np.complex128)
    ga, gb, gg = _dev(torch, A), _dev(torch, B), _dev(torch, G)
    da, db = torch.empty_like(ga), torch.empty_like(gb)
    v = lambda x: t1m.tensor(list(x.shape), x, t1m.row_major)  # noqa: E731
    t1m.contract_vjp(v(gg), lc, v(ga), la, v(gb), lb, v(da), v(db), ctx=ctx)
    dA, dB = da.cpu().numpy(), db.cpu().numpy()

    def loss(a, b):
        out = torch.empty([ext[c] for c in lc], dtype=torch.complex128, device="cuda")
        t1m.contract_raw(1.0, v(_dev(torch, a)), la, v(_dev(torch, b)), lb, 0.0, v(out), lc, 0,
                         ctx)
        return float(np.real(np.sum(np.conj(G) * out.cpu().numpy())))

    h = 1e-6
    for _ in range(3):
        VA = _rand(rng, A.shape, np.complex128)
        VB = _rand(rng, B.shape, np.complex128)
        fd_a = (loss(A + h * VA, B) - loss(A - h * VA, B)) / (2 * h)
        fd_b = (loss(A, B + h * VB) - loss(A, B - h * VB)) / (2 * h)
        an_a = float(np.real(np.sum(np.conj(dA) * VA)))
        an_b = float(np.real(np.sum(np.conj(dB) * VB)))
        assert abs(fd_a - an_a) <= 1e-7 * max(1.0, abs(an_a))
        assert abs(fd_b - an_b) <= 1e-7 * max(1.0, abs(an_b))


def test_gradcheck_autograd_wrapper(torch_cuda):
    torch = torch_cuda
    from autograd_fn import contract
    rng = np.random.default_rng(10)
    a = _dev(torch, _rand(rng, (3, 4, 2), np.complex128)).requires_grad_(True)
    b = _dev(torch, _rand(rng, (4, 5), np.complex128)).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda x, y: contract(x, y, "abc", "bd", "acd", "plain"),
                                    (a, b), eps=1e-6, atol=1e-7, rtol=1e-6)


RING = (["apb", "bpc", "cqd", "dqa"], ["ac", "aqd", ""])


@pytest.mark.parametrize("bond,phys", [(8, 2), (64, 8)])
def test_ring_chain_gradients(ctx, torch_cuda, bond, phys):
    """Ring of four order-3 tensors contracted to a scalar; gradients of
    Re(s) from the recomputing chain vs directional central differences
    (complex128) and vs torch autograd of einsum (complex128)."""
    import t1m_gb300 as t1m
    from t1m_gb300.chain import ContractionChain
    torch = torch_cuda
    rng = np.random.default_rng(11)
    labels, outs = RING
    ext = dict(a=bond, b=bond, c=bond, d=bond, p=phys, q=phys)
    scale = 1.0 / np.sqrt(bond)
    xs = [_dev(torch, scale * _rand(rng, [ext[c] for c in lab], np.complex128)) for lab in labels]
    chain = ContractionChain(labels, outs)
    s = chain.forward(xs, ctx=ctx)
    assert s.dim() == 0
    one = torch.ones((), dtype=torch.complex128, device="cuda")
    grads = chain.backward(xs, one, ctx=ctx)
    # torch einsum autograd as an independent check.
    ts = [x.clone().requires_grad_(True) for x in xs]
    s_t = torch.einsum("apb,bpc,cqd,dqa->", *ts)
    s_t.real.backward()
    s_ref = complex(s_t.detach().cpu())
    assert abs(complex(s.cpu()) - s_ref) <= 1e-10 * max(1, abs(s_ref))
    for g, t in zip(grads, ts):
        ref = t.grad
        assert (g - ref).abs().max().item() <= 1e-10 * max(1.0, ref.abs().max().item())
    # Directional finite differences on the first and last tensors.
    h = 1e-6
    for i in (0, 3):
        V = _dev(torch, _rand(rng, list(xs[i].shape), np.complex128))
        xp = list(xs)
        xm = list(xs)
        xp[i] = xs[i] + h * V
        xm[i] = xs[i] - h * V
        fd = (chain.forward(xp, ctx=ctx).real - chain.forward(xm, ctx=ctx).real).item() / (2 * h)
        an = torch.sum(torch.conj(grads[i]) * V).real.item()
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an))


def test_ring_chain_complex64_tensor_cores_vs_complex128(ctx, torch_cuda):
    """The same ring in complex64 on the tensor cores: value and gradients
    within 1e-5 (normwise) of the complex128 chain."""
    from t1m_gb300.chain import ContractionChain
    torch = torch_cuda
    rng = np.random.default_rng(12)
    labels, outs = RING
    ext = dict(a=64, b=64, c=64, d=64, p=8, q=8)
    xs = [_dev(torch, _rand(rng, [ext[c] for c in lab], np.complex128) / 8.0) for lab in labels]
    chain = ContractionChain(labels, outs)
    one = torch.ones((), dtype=torch.complex128, device="cuda")
    g128 = chain.backward(xs, one, ctx=ctx)
    xs64 = [x.to(torch.complex64) for x in xs]
    ctx.set_method("tc_3xtf32")
    try:
        g64 = chain.backward(xs64, one.to(torch.complex64), ctx=ctx)
    finally:
        ctx.set_method("auto")
    for a, b in zip(g64, g128):
        err = (a.to(torch.complex128) - b).abs().max().item() / b.abs().max().item()
        assert err < 1e-5, err


@pytest.mark.parametrize("dt,bond,phys", [("complex128", 8, 2), ("complex128", 64, 8),
                                          ("complex64", 64, 8)])
def test_ring_chain_grouped_mode(ctx, torch_cuda, dt, bond, phys):
    """The chain as one grouped launch per pass (intermediates kept in device
    memory, adjoint products as conjugating group items): forward value and
    gradients equal the recomputing chain's and torch autograd's, and replays
    of the planned groups give the same results."""
    from t1m_gb300.chain import ContractionChain
    torch = torch_cuda
    rng = np.random.default_rng(13)
    labels, outs = RING
    ext = dict(a=bond, b=bond, c=bond, d=bond, p=phys, q=phys)
    scale = 1.0 / np.sqrt(bond)
    xs = [_dev(torch, scale * _rand(rng, [ext[c] for c in lab], np.complex128)).to(
        getattr(torch, dt)) for lab in labels]
    one = torch.ones((), dtype=xs[0].dtype, device="cuda")
    ref_chain = ContractionChain(labels, outs)
    s_ref = complex(ref_chain.forward(xs, ctx=ctx).cpu())
    g_ref = ref_chain.backward(xs, one, ctx=ctx)
    chain = ContractionChain(labels, outs, mode="grouped")
    tol = 1e-10 if dt == "complex128" else 2e-5
    try:
        for _ in range(2):  # first call plans the groups, the second replays them
            s = complex(chain.forward(xs, ctx=ctx).cpu())
            grads = [g.clone() for g in chain.backward(xs, one, ctx=ctx)]
            assert abs(s - s_ref) <= tol * max(1.0, abs(s_ref)), (s, s_ref)
            for g, r in zip(grads, g_ref):
                err = (g.to(torch.complex128) - r.to(torch.complex128)).abs().max().item()
                assert err <= tol * max(1.0, r.abs().max().item()), err
    finally:
        chain.close()
    # torch autograd of einsum in complex128 as an independent check.
    ts = [x.to(torch.complex128).clone().requires_grad_(True) for x in xs]
    torch.einsum("apb,bpc,cqd,dqa->", *ts).real.backward()
    for g, t in zip(grads, ts):
        err = (g.to(torch.complex128) - t.grad).abs().max().item()
        assert err <= max(tol, 1e-5 if dt == "complex64" else 1e-10) * max(1.0, t.grad.abs().max().item())
