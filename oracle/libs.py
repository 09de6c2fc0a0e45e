"""ctypes access to the oracle libraries (test infrastructure only).

``port_contract`` calls the C++ restatement (oracle/port/t1m_port.cpp);
``ref_*`` call the unmodified reference through oracle/ref_shim.cpp when that
shim was built here (it only exists where the reference tree exists).
"""
from __future__ import annotations

import ctypes as C
from functools import lru_cache

import numpy as np

from . import build as _build

DTYPE_CODE = {np.dtype(np.float32): 0, np.dtype(np.float64): 1,
              np.dtype(np.complex64): 2, np.dtype(np.complex128): 3}

_i64p = C.POINTER(C.c_int64)
_lp = C.POINTER(C.c_long)


@lru_cache(maxsize=None)
def port_lib() -> C.CDLL:
    lib = C.CDLL(str(_build.build_port()))
    lib.t1m_port_contract.restype = C.c_int
    lib.t1m_port_contract.argtypes = [
        C.c_int,
        C.c_int, _i64p, _i64p, C.c_void_p, C.c_char_p,
        C.c_int, _i64p, _i64p, C.c_void_p, C.c_char_p,
        C.c_int, _i64p, _i64p, C.c_void_p, C.c_char_p,
        C.c_void_p, C.c_void_p, C.c_int]
    return lib


@lru_cache(maxsize=None)
def ref_lib() -> C.CDLL | None:
    path = _build.build_ref()
    if path is None or not path.exists():
        return None
    lib = C.CDLL(str(path))
    lib.t1mref_contract.restype = C.c_int
    lib.t1mref_contract.argtypes = [
        C.c_int, C.c_int, _lp, C.c_void_p, C.c_char_p, C.c_int, _lp, C.c_void_p,
        C.c_char_p, C.c_int, _lp, C.c_void_p, C.c_char_p, C.c_double, C.c_double]
    lib.t1mref_index_bundles.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, _lp,
                                         C.POINTER(C.c_int)]
    lib.t1mref_scatter.restype = C.c_long
    lib.t1mref_scatter.argtypes = [C.c_int, _lp, _lp, C.c_int, _lp, _lp]
    lib.t1mref_block_scatter.restype = C.c_long
    lib.t1mref_block_scatter.argtypes = [_lp, C.c_long, C.c_long, _lp]
    lib.t1mref_pack_block.argtypes = [C.c_int, C.c_int, C.c_int, _lp, C.c_int, _lp,
                                      C.c_int, _lp, C.c_long, C.c_long, C.c_long,
                                      C.c_void_p, C.c_void_p]
    lib.t1mref_unpack.argtypes = [C.c_int, C.c_int, _lp, C.c_int, _lp, C.c_int, _lp,
                                  C.c_long, C.c_long, C.c_void_p, C.c_void_p]
    return lib


def _arr64(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.int64))
    return a, a.ctypes.data_as(_i64p)


def _arrl(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.int64))
    return a, a.ctypes.data_as(_lp)


def _flat_extent(dims, strides) -> int:
    return 1 + sum((int(d) - 1) * int(s) for d, s in zip(dims, strides))


def port_contract(flat_a, dims_a, strides_a, la, flat_b, dims_b, strides_b, lb,
                  flat_c, dims_c, strides_c, lc, alpha=1.0, beta=0.0,
                  nthreads=1):
    """Run the port in place on flat element buffers (C is updated: the
    reference's C <- C + alpha*A*B, or C + A*B for complex)."""
    assert flat_a.dtype == flat_b.dtype == flat_c.dtype
    assert flat_c.flags.c_contiguous
    for f, d, s in ((flat_a, dims_a, strides_a), (flat_b, dims_b, strides_b),
                    (flat_c, dims_c, strides_c)):
        assert f.size >= _flat_extent(d, s)
    code = DTYPE_CODE[flat_a.dtype]
    real_t = np.float32 if code in (0, 2) else np.float64
    al = np.array([alpha], dtype=real_t)
    be = np.array([beta], dtype=real_t)
    keep = []
    args = []
    for f, d, s, lab in ((flat_a, dims_a, strides_a, la), (flat_b, dims_b, strides_b, lb),
                         (flat_c, dims_c, strides_c, lc)):
        da, pda = _arr64(d)
        sa, psa = _arr64(s)
        keep += [da, sa]
        args += [len(d), pda, psa, f.ctypes.data, lab.encode()]
    rc = port_lib().t1m_port_contract(code, *args, al.ctypes.data, be.ctypes.data,
                                      int(nthreads))
    if rc != 0:
        raise ValueError(f"t1m_port_contract failed ({rc})")
    return flat_c


def ref_contract(flat_a, dims_a, la, flat_b, dims_b, lb, flat_c, dims_c, lc,
                 alpha=1.0, beta=0.0):
    """Run the unmodified reference (column-major tensors) in place on C."""
    lib = ref_lib()
    if lib is None:
        raise RuntimeError("reference shim not built (reference tree absent)")
    code = DTYPE_CODE[flat_a.dtype]
    keep, args = [], []
    for f, d, lab in ((flat_a, dims_a, la), (flat_b, dims_b, lb), (flat_c, dims_c, lc)):
        da, pda = _arrl(d)
        keep.append(da)
        args += [len(d), pda, f.ctypes.data, lab.encode()]
    rc = lib.t1mref_contract(code, *args, float(alpha), float(beta))
    if rc != 0:
        raise ValueError(f"t1mref_contract failed ({rc})")
    return flat_c


def ref_index_bundles(la, lb, lc):
    lib = ref_lib()
    out = np.zeros(96, dtype=np.int64)
    counts = (C.c_int * 6)()
    lib.t1mref_index_bundles(la.encode(), lb.encode(), lc.encode(),
                             out.ctypes.data_as(_lp), counts)
    names = ["AX", "AY", "BX", "BY", "CX", "CY"]
    return {n: [int(v) for v in out[16 * i:16 * i + counts[i]]] for i, n in enumerate(names)}


def ref_scatter(indices, dims, strides):
    lib = ref_lib()
    n = 1
    for i in indices:
        n *= int(dims[i])
    out = np.zeros(max(n, 1), dtype=np.int64)
    d, pd = _arrl(dims)
    s, ps = _arrl(strides)
    ix, pix = _arrl(indices)
    m = lib.t1mref_scatter(len(dims), pd, ps, len(indices), pix, out.ctypes.data_as(_lp))
    return out[:m]


def ref_block_scatter(scat, b):
    lib = ref_lib()
    s, ps = _arrl(scat)
    out = np.zeros(len(s) // b + 2, dtype=np.int64)
    m = lib.t1mref_block_scatter(ps, len(s), int(b), out.ctypes.data_as(_lp))
    return out[:m]


def ref_pack_block(src, dims, bx, by, br, bc, length, label, dest_len):
    lib = ref_lib()
    src = np.ascontiguousarray(src)
    code = 2 if np.iscomplexobj(src) else 0
    dest = np.zeros(dest_len, dtype=np.float32)
    d, pd = _arrl(dims)
    x, px = _arrl(bx)
    y, py = _arrl(by)
    rc = lib.t1mref_pack_block(code, 0 if label == "A" else 1, len(dims), pd, len(bx), px,
                               len(by), py, br, bc, length, src.ctypes.data,
                               dest.ctypes.data)
    assert rc == 0
    return dest


def ref_unpack(src, dims, bx, by, br, bc, dest):
    lib = ref_lib()
    src = np.ascontiguousarray(src)
    dest = np.array(dest, copy=True)
    code = 2 if np.iscomplexobj(dest) else 0
    d, pd = _arrl(dims)
    x, px = _arrl(bx)
    y, py = _arrl(by)
    rc = lib.t1mref_unpack(code, len(dims), pd, len(bx), px, len(by), py, br, bc,
                           src.ctypes.data, dest.ctypes.data)
    assert rc == 0
    return dest
