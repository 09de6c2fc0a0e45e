"""t1m_contract_noalloc, the entry point for callers that cannot allocate
device memory (their own memory pool owns the GPU, or allocation and the
device-wide synchronisation of cudaFree are not acceptable where they call
from).  It must give the same results as t1m_contract, within the tolerances
of the FP64 oracle, while using only the library's fixed scratch array and
allocating nothing.

Collected last on purpose (file name), so a run that stops at the first
failure has already run every other test; it also passes alone in a fresh
process."""
import ctypes as C

import numpy as np
import pytest

from oracle import numpy_oracle as no

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 64 << 20  # T1M_NOALLOC_SCRATCH_BYTES

CASES = [
    # labels, extents, dtype, method: the first splits K (partial products in
    # the scratch array), the others exercise other kernels and dtypes, and
    # the automatic method (tensor cores for complex64 and float32 here).
    (("abcd", "dbea", "ec"), dict(a=12, b=16, c=96, d=24, e=64), np.complex64, "tc_3xtf32"),
    (("abcd", "dbea", "ec"), dict(a=12, b=16, c=96, d=24, e=64), np.complex64, "plain"),
    (("abcd", "efcd", "abef"), dict(a=20, b=12, c=16, d=9, e=24, f=10), np.complex128, "dmma"),
    (("ab", "bc", "ac"), dict(a=300, b=700, c=200), np.float32, "plain"),
    (("mk", "kn", "mn"), dict(m=256, k=256, n=256), np.complex64, "auto"),
    (("ab", "bc", "ac"), dict(a=300, b=700, c=200), np.float32, "auto"),
]


def _tol(dt):
    return 1e-12 if np.dtype(dt) in (np.float64, np.complex128) else 2e-5


def _dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def _noalloc(t1m, torch, method, alpha, ta, la, tb, lb, beta, tc, lc):
    """One call through the C-ABI; returns (status, message)."""
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
    return st, err.value.decode()


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0][0]}-{c[3]}-{np.dtype(c[2]).name}")
def test_noalloc_matches_contract_and_fp64_twice(case):
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

    # The FP64 oracle (column-major views of the flat buffers).
    cm = no.col_major_strides
    ref64 = no.contract_fp64(no.as_strided_view(A, da, cm(da)), la,
                             no.as_strided_view(B, db, cm(db)), lb,
                             no.as_strided_view(C0, dc, cm(dc)), lc, alpha, beta)
    ref64 = np.asarray(ref64).reshape(-1, order="F")

    # The existing entry point.
    ctx = t1m.Context()
    ctx.set_method(method)
    g_ref = _dev(torch, C0)
    rep = t1m.contract_scaled(alpha, ta, la, tb, lb, beta, t1m.tensor(dc, g_ref), lc, ctx=ctx)
    torch.cuda.synchronize()
    ref = g_ref.cpu().numpy().astype(np.complex128)
    ctx.close()

    tol = _tol(dt)
    assert no.rel_errors(ref, ref64)[0] < tol
    outs = [_dev(torch, C0) for _ in range(3)]
    st, msg = _noalloc(t1m, torch, method, alpha, ta, la, tb, lb, beta, t1m.tensor(dc, outs[0]), lc)
    assert st == 0, msg
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for g_out in outs[1:]:  # two calls in a row share (and overwrite) the scratch
        st, msg = _noalloc(t1m, torch, method, alpha, ta, la, tb, lb, beta,
                           t1m.tensor(dc, g_out), lc)
        assert st == 0, msg
        got = g_out.cpu().numpy().astype(np.complex128)
        scale = np.abs(ref).max()
        assert np.abs(got - ref).max() / scale < tol
        assert no.rel_errors(got, ref64)[0] < tol
    # No device memory was taken by the calls after the first (which may
    # load kernel modules).
    assert torch.cuda.mem_get_info()[0] == free0
    if case is CASES[0]:
        assert rep.split_k > 1  # the scratch holds split-K partials here


def test_noalloc_split_shrinks_to_fit_scratch():
    """complex128 DMMA, 32 x 64 output, K = 2^21 (a 16 x 131072 contracted
    bundle over overlapping strides, so the operands stay small): its scatter
    vectors take half the scratch, the automatic split count (1216 partials,
    40 MB) does not fit the rest and shrinks.  Checked against FP64 and
    against t1m_contract (whose workspace takes all 1216)."""
    import torch
    import t1m_gb300 as t1m
    M, N, K1, K2 = 32, 64, 16, 131072
    gen = torch.Generator(device="cuda")
    gen.manual_seed(3)

    def mk(n):
        return torch.complex(torch.rand(n, device="cuda", generator=gen, dtype=torch.float64) * 2 - 1,
                             torch.rand(n, device="cuda", generator=gen, dtype=torch.float64) * 2 - 1)

    a_str, b_str = (1, M, 1), (1, 1, K1)
    ga = mk((M - 1) + (K1 - 1) * M + (K2 - 1) + 1)
    gb = mk((K1 - 1) + (K2 - 1) + (N - 1) * K1 + 1)
    vec_bytes = 8 * (2 * M + 2 * N + 2 * K1 * K2)
    assert SCRATCH_BYTES // 2 < vec_bytes < SCRATCH_BYTES
    ta = t1m.tensor([M, K1, K2], ga, strides=a_str)
    tb = t1m.tensor([K1, K2, N], gb, strides=b_str)
    la, lb, lc = "mkl", "kln", "mn"
    ref = (ga.as_strided((M, K1, K2), a_str).reshape(M, -1) @
           gb.as_strided((K1, K2, N), b_str).reshape(-1, N)).t().reshape(-1)  # col-major C
    ctx = t1m.Context()
    ctx.set_method("dmma")
    gc = torch.zeros(M * N, dtype=torch.complex128, device="cuda")
    rep = t1m.contract_scaled(1.0, ta, la, tb, lb, 0.0, t1m.tensor([M, N], gc), lc, ctx=ctx)
    torch.cuda.synchronize()
    ctx.close()
    assert rep.split_k * M * N * 16 > SCRATCH_BYTES - vec_bytes
    scale = ref.abs().max().item()
    assert (gc - ref).abs().max().item() / scale < 1e-12
    for _ in range(2):
        out = torch.zeros_like(gc)
        st, msg = _noalloc(t1m, torch, "dmma", 1.0, ta, la, tb, lb, 0.0, t1m.tensor([M, N], out), lc)
        assert st == 0, msg
        assert (out - ref).abs().max().item() / scale < 1e-12
        assert (out - gc).abs().max().item() / scale < 1e-12


def test_noalloc_rejects_scatter_vectors_beyond_scratch():
    """M = 2^22 rows: A's and C's row offsets alone (2 x 32 MiB) exceed the
    scratch, so the call is refused with T1M_ERR_UNSUPPORTED before any
    launch."""
    import torch
    import t1m_gb300 as t1m
    M = 1 << 22
    ga = torch.zeros(M, dtype=torch.complex64, device="cuda")
    gb = torch.ones(1, dtype=torch.complex64, device="cuda")
    gc = torch.zeros(M, dtype=torch.complex64, device="cuda")
    st, msg = _noalloc(t1m, torch, "auto", 1.0, t1m.tensor([M, 1], ga), "mk",
                       t1m.tensor([1, 1], gb), "kn", 0.0, t1m.tensor([M, 1], gc), "mn")
    assert st == 5 and "scratch" in msg, (st, msg)


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
