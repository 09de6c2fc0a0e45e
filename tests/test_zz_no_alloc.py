"""t1m_contract_noalloc, the entry point for callers that cannot allocate
device memory (their own memory pool owns the GPU, or allocation and the
device-wide synchronisation of cudaFree are not acceptable where they call
from).  It must give the same results as t1m_contract while using only the
library's fixed scratch array.

Collected last on purpose (file name), so a run that stops at the first
failure has already run every other test; it also passes alone in a fresh
process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    # labels, extents, dtype, method: the first splits K (partial products in
    # the scratch array), the others exercise other kernels and dtypes.
    (("abcd", "dbea", "ec"), dict(a=12, b=16, c=96, d=24, e=64), np.complex64, "tc_3xtf32"),
    (("abcd", "dbea", "ec"), dict(a=12, b=16, c=96, d=24, e=64), np.complex64, "plain"),
    (("abcd", "efcd", "abef"), dict(a=20, b=12, c=16, d=9, e=24, f=10), np.complex128, "dmma"),
    (("ab", "bc", "ac"), dict(a=300, b=700, c=200), np.float32, "plain"),
]


def _dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def _noalloc(t1m, torch, method, alpha, ta, la, tb, lb, beta, tc, lc):
    keep = []
    ca, cb, cc = ta._c(keep), tb._c(keep), tc._c(keep)
    dtype = t1m._DTYPE_OF[tc.dtype()]
    al, be = t1m._scalar_bytes(dtype, alpha), t1m._scalar_bytes(dtype, beta)
    err = C.create_string_buffer(512)
    stream = torch.cuda.current_stream().cuda_stream
    st = t1m.lib().t1m_contract_noalloc(stream, int(t1m.method[method]), dtype,
                                        C.cast(al, C.c_void_p), C.byref(ca), la.encode(),
                                        C.byref(cb), lb.encode(), C.cast(be, C.c_void_p),
                                        C.byref(cc), lc.encode(), 0, err, 512)
    assert st == 0, err.value.decode()


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0][0]}-{c[3]}-{np.dtype(c[2]).name}")
def test_noalloc_matches_contract_twice(case):
    import torch
    import t1m_gb300 as t1m
    (la, lb, lc), ext, dt, method = case
    da, db, dc = ([ext[ch] for ch in s] for s in (la, lb, lc))
    rng = np.random.default_rng(21)

    def r(shape):
        x = rng.uniform(-1, 1, shape)
        if np.dtype(dt).kind == "c":
            x = x + 1j * rng.uniform(-1, 1, shape)
        return x.astype(dt)

    A, B, C0 = r(int(np.prod(da))), r(int(np.prod(db))), r(int(np.prod(dc)))
    alpha = (1 + 0.5j) if np.dtype(dt).kind == "c" else 1.5
    beta = 0.25
    ga, gb = _dev(torch, A), _dev(torch, B)
    ta, tb = t1m.tensor(da, ga), t1m.tensor(db, gb)

    # The existing entry point.
    ctx = t1m.Context()
    ctx.set_method(method)
    g_ref = _dev(torch, C0)
    rep = t1m.contract_scaled(alpha, ta, la, tb, lb, beta, t1m.tensor(dc, g_ref), lc, ctx=ctx)
    torch.cuda.synchronize()
    ref = g_ref.cpu().numpy().astype(np.complex128)
    ctx.close()

    tol = 1e-12 if np.dtype(dt) in (np.float64, np.complex128) else 2e-5
    scale = np.abs(ref).max()
    for _ in range(2):  # two calls in a row share (and overwrite) the scratch
        g_out = _dev(torch, C0)
        _noalloc(t1m, torch, method, alpha, ta, la, tb, lb, beta, t1m.tensor(dc, g_out), lc)
        got = g_out.cpu().numpy().astype(np.complex128)
        assert np.abs(got - ref).max() / scale < tol
    if case is CASES[0]:
        assert rep.split_k > 1  # the scratch holds split-K partials here


def test_noalloc_rejects_host_pointers():
    import t1m_gb300 as t1m
    import torch
    A, B, Cm = (np.ones(6, np.complex64), np.ones(6, np.complex64), np.zeros(4, np.complex64))
    keep = []
    ca = t1m.tensor([2, 3], A)._c(keep)
    cb = t1m.tensor([3, 2], B)._c(keep)
    cc = t1m.tensor([2, 2], Cm)._c(keep)
    one = t1m._scalar_bytes(t1m.COMPLEX64, 1.0)
    err = C.create_string_buffer(256)
    st = t1m.lib().t1m_contract_noalloc(torch.cuda.current_stream().cuda_stream, 0,
                                        t1m.COMPLEX64, C.cast(one, C.c_void_p), C.byref(ca),
                                        b"ab", C.byref(cb), b"bc", C.cast(one, C.c_void_p),
                                        C.byref(cc), b"ac", 0, err, 256)
    assert st == 1 and b"device pointers" in err.value
