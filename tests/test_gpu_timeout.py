"""The bounded-wait timeout path of the persistent tensor-core kernel (gpu).

The failure is made on the host: T1M_GROUP_INJECT_UNMET_DEPENDENCY makes every
dependent item of a single persistent launch wait for one more tile than its
dependency writes, a count that nothing reaches.  With a 1 ms wait limit the
dependent tiles give up, set the error word and drain their remaining stages
without loads, so every MMA pipeline runs to its end (no MMA-side wait runs
out) and TMEM is freed normally.  The launch must report
T1M_ERR_KERNEL_TIMEOUT quickly, and the same context must then run correct
contractions and groups.  No GPU fault is involved."""
import time

import numpy as np
import pytest

from oracle import numpy_oracle as no

pytestmark = pytest.mark.gpu

TIMEOUT_STATUS = 6  # T1M_ERR_KERNEL_TIMEOUT


def _items(torch, t1m, rng, n=3):
    """All-tensor-core chain pairs (one persistent launch with in-kernel
    dependencies): R = X1 X2, then O = R X3."""
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    items, checks = [], []
    for _ in range(n):
        x, a, q = (int(val) for val in rng.choice([32, 64, 96], 3))
        X1 = (rng.uniform(-1, 1, (x, a)) + 1j * rng.uniform(-1, 1, (x, a))).astype(np.complex64)
        X2 = (rng.uniform(-1, 1, (a, 64)) + 1j * rng.uniform(-1, 1, (a, 64))).astype(np.complex64)
        X3 = (rng.uniform(-1, 1, (64, q)) + 1j * rng.uniform(-1, 1, (64, q))).astype(np.complex64)
        g1, g2, g3 = (torch.from_numpy(z.copy()).cuda() for z in (X1, X2, X3))
        r = torch.zeros((x, 64), dtype=torch.complex64, device="cuda")
        o = torch.zeros((x, q), dtype=torch.complex64, device="cuda")
        i1 = len(items)
        items.append((1.0, v(g1), "xa", v(g2), "ay", 0.0, v(r), "xy", -1))
        items.append((1.0, v(r), "xy", v(g3), "yq", 0.0, v(o), "xq", i1))
        checks.append((X1, X2, X3, r, o, (g1, g2, g3)))
    return items, checks


def _check(checks):
    for X1, X2, X3, r, o, _ in checks:
        R = X1.astype(np.complex128) @ X2.astype(np.complex128)
        O = R @ X3.astype(np.complex128)
        for got, want in ((r, R), (o, O)):
            mx, _ = no.rel_errors(got.cpu().numpy(), want)
            assert mx < 2e-6, mx


@pytest.mark.parametrize("graph", [False, True])
def test_unmet_dependency_times_out_and_context_recovers(ctx, torch_cuda, graph):
    import t1m_gb300 as t1m
    torch = torch_cuda
    rng = np.random.default_rng(41)
    items, checks = _items(torch, t1m, rng)
    ctx.set_wait_limit(1000)  # 1 ms
    try:
        bad = t1m.Group(items, ctx=ctx, graph=graph,
                        options=t1m.GROUP_INJECT_UNMET_DEPENDENCY)
        t0 = time.perf_counter()
        with pytest.raises(t1m.T1MError) as exc:
            bad.launch(timed=True)
        elapsed = time.perf_counter() - t0
        bad.close()
    finally:
        ctx.set_wait_limit(0)
    assert exc.value.status == TIMEOUT_STATUS, exc.value
    assert elapsed < 1.0, elapsed  # bounded by the 1 ms limit, not the default 2 s

    # The context is usable: the same batch without the injected count, and
    # a single contraction, give correct results.
    good = t1m.Group(items, ctx=ctx, graph=graph)
    rep = good.launch(timed=True)
    assert rep.kernels == 1
    good.close()
    _check(checks)
    A = (rng.uniform(-1, 1, (256, 256)) + 1j * rng.uniform(-1, 1, (256, 256))).astype(np.complex64)
    ga = torch.from_numpy(A).cuda()
    gc = torch.zeros_like(ga)
    t1m.contract_scaled(1.0, t1m.tensor([256, 256], ga), "mk", t1m.tensor([256, 256], ga), "kn",
                        0.0, t1m.tensor([256, 256], gc), "mn", ctx=ctx)
    # Column-major views of row-major buffers: the buffer of C holds A @ A.
    A64 = A.astype(np.complex128)
    assert no.rel_errors(gc.cpu().numpy().reshape(256, 256), A64 @ A64)[0] < 1e-6
