"""t1m_gb300 — Python host API over libt1m_cuda.so (the C-ABI of include/t1m_capi.h).

Mirrors the reference's public interface (include/t1m/t1m.h):

* ``memory_layout`` with ``row_major`` / ``col_major`` (t1m.h:29),
* ``tensor(dims, data, layout=col_major)`` — a non-owning view (t1m.h:31-66),
* ``contract(a, "abc", b, "bd", c, "acd")`` for complex tensors and
  ``contract(alpha, a, la, b, lb, beta, c, lc)`` for real ones (t1m.h:560-577),
  with the reference's semantics C <- C + alpha*A*B,

plus ``contract_scaled`` (C <- alpha*A*B + beta*C with complex alpha/beta) and
the adjoint ``contract_vjp``.  Data may be numpy arrays (host memory, staged by
the library) or torch tensors / raw device pointers (used in place).

The compute always runs in libt1m_cuda.so on the GPU; there is no CPU path.
If the library is missing this module raises instead of falling back.
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass
from pathlib import Path
from typing import Any, Sequence

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libt1m_cuda.so"

# t1m_status
OK = 0
_STATUS = {1: "invalid argument", 2: "invalid labels or extents", 3: "allocation failed",
           4: "CUDA error", 5: "unsupported method", 6: "device-side wait timed out",
           7: "no usable CUDA device"}

# t1m_dtype
FLOAT32, FLOAT64, COMPLEX64, COMPLEX128 = 0, 1, 2, 3
_NP_DTYPE = {FLOAT32: np.float32, FLOAT64: np.float64, COMPLEX64: np.complex64,
             COMPLEX128: np.complex128}
_DTYPE_OF = {np.dtype(v): k for k, v in _NP_DTYPE.items()}

FLAG_ACCUMULATE = 1
FLAG_CONJ_A = 2
FLAG_CONJ_B = 4
FLAG_NO_TIMING = 8


# t1m_report.path (T1M_PATH_* of t1m_capi.h)
PATH_TC, PATH_PERSISTENT, PATH_A_PACKED, PATH_B_PACKED = 0x1000, 0x100, 0x200, 0x400
PATH_PAIR = 0x800
PATH_PIECES = 0x2000
# t1m_set_tile_form
TILE_FORMS = {"auto": 0, "one": 1, "pair": 2, "pieces": 3}
A_MODES = {0: "gather", 1: "MK", 2: "MK16", 3: "KM", 4: "KM16", 5: "MK16K"}
B_MODES = {0: "gather", 1: "NK", 2: "KN", 3: "NK16", 4: "KN16", 5: "panels"}


class memory_layout(enum.IntEnum):
    """Same values as the reference's enum (t1m.h:29)."""
    row_major = 0
    col_major = 1


row_major = memory_layout.row_major
col_major = memory_layout.col_major
STRIDED = 2


class method(enum.IntEnum):
    auto = 0
    plain = 1
    tc_3xtf32 = 2
    tc_bf16x3 = 3
    tc_bf16x6 = 4
    dmma = 5


class T1MError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"t1m status {status} ({_STATUS.get(status, '?')}): {message}")
        self.status = status


class _Tensor(C.Structure):
    _fields_ = [("ndim", C.c_int32), ("layout", C.c_int32),
                ("extents", C.POINTER(C.c_int64)), ("strides", C.POINTER(C.c_int64)),
                ("data", C.c_void_p)]


class Report(C.Structure):
    _fields_ = [("method", C.c_int32), ("split_k", C.c_int32), ("m", C.c_int64),
                ("n", C.c_int64), ("k", C.c_int64), ("flops", C.c_double),
                ("kernel_ms", C.c_double), ("h2d_ms", C.c_double), ("d2h_ms", C.c_double),
                ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64), ("kernels", C.c_int32),
                ("path", C.c_int32), ("main_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}

    @property
    def fetch(self) -> dict | None:
        """How the last tensor-core product fetched its operands (decoded
        t1m_report.path; None for the plain and FP64 kernels)."""
        p = self.path
        if not p & PATH_TC:
            return None
        return {"a": A_MODES[p & 15], "b": B_MODES[(p >> 4) & 15],
                "persistent": bool(p & PATH_PERSISTENT), "pair": bool(p & PATH_PAIR),
                "pieces": bool(p & PATH_PIECES), "a_packed": bool(p & PATH_A_PACKED),
                "b_packed": bool(p & PATH_B_PACKED)}


class PlanInfo(C.Structure):
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("k", C.c_int64), ("modes_m", C.c_int32),
                ("modes_n", C.c_int32), ("modes_k", C.c_int32), ("reserved", C.c_int32)]


class GroupItem(C.Structure):
    _fields_ = [("a", C.POINTER(_Tensor)), ("labels_a", C.c_char_p),
                ("b", C.POINTER(_Tensor)), ("labels_b", C.c_char_p),
                ("c", C.POINTER(_Tensor)), ("labels_c", C.c_char_p),
                ("alpha", C.c_double * 2), ("beta", C.c_double * 2),
                ("depends_on", C.c_int32), ("flags", C.c_uint32)]


GROUP_GRAPH = 1
GROUP_AUTOTUNE = 2
GROUP_INJECT_UNMET_DEPENDENCY = 4
GROUP_ONE_LAUNCH = 8
GROUP_TILE_16, GROUP_TILE_32, GROUP_TILE_64, GROUP_TILE_128 = 16, 32, 64, 128

_lib_handle: C.CDLL | None = None


def lib() -> C.CDLL:
    """Load libt1m_cuda.so (raises if it was not built)."""
    global _lib_handle
    if _lib_handle is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"`"
                " (t1m_gb300 has no CPU fallback)")
        h = C.CDLL(str(LIB_PATH))
        vp, i32, u32 = C.c_void_p, C.c_int, C.c_uint32
        h.t1m_create.argtypes = [C.POINTER(vp), i32]
        h.t1m_destroy.argtypes = [vp]
        h.t1m_set_stream.argtypes = [vp, vp]
        h.t1m_set_method.argtypes = [vp, i32]
        h.t1m_set_split_k.argtypes = [vp, i32]
        h.t1m_set_workspace_limit.argtypes = [vp, C.c_int64]
        h.t1m_set_tile_form.argtypes = [vp, i32]
        h.t1m_set_wait_limit.argtypes = [vp, C.c_int64]
        h.t1m_set_autotune.argtypes = [vp, i32]
        h.t1m_synchronize.argtypes = [vp]
        h.t1m_status_string.restype = C.c_char_p
        h.t1m_status_string.argtypes = [i32]
        h.t1m_last_error.restype = C.c_char_p
        h.t1m_last_error.argtypes = [vp]
        h.t1m_version.argtypes = [C.POINTER(C.c_int)] * 3
        tp = C.POINTER(_Tensor)
        h.t1m_contract.argtypes = [vp, i32, vp, tp, C.c_char_p, tp, C.c_char_p, vp, tp,
                                   C.c_char_p, u32, C.POINTER(Report)]
        h.t1m_analyze.argtypes = [i32, tp, C.c_char_p, tp, C.c_char_p, tp, C.c_char_p,
                                  C.POINTER(PlanInfo), C.c_char_p, C.c_int32]
        h.t1m_contract_noalloc.argtypes = [vp, i32, i32, vp, tp, C.c_char_p, tp, C.c_char_p,
                                           vp, tp, C.c_char_p, u32, C.c_char_p, C.c_int32]
        h.t1m_contract_vjp.argtypes = [vp, i32, tp, C.c_char_p, tp, C.c_char_p, tp, C.c_char_p,
                                       tp, tp, u32, C.POINTER(Report)]
        h.t1m_group_create.argtypes = [vp, i32, i32, C.POINTER(GroupItem), u32, C.POINTER(vp)]
        h.t1m_group_launch.argtypes = [vp, C.POINTER(Report)]
        h.t1m_group_destroy.argtypes = [vp]
        _lib_handle = h
    return _lib_handle


class Context:
    """The C-ABI context (replaces the reference's BLIS cntx_t* slot)."""

    def __init__(self, device: int = 0, method_: int | str = method.auto):
        self._h = C.c_void_p()
        st = lib().t1m_create(C.byref(self._h), int(device))
        if st != OK:
            raise T1MError(st, "t1m_create failed")
        self.set_method(method_)

    def set_method(self, m: int | str) -> None:
        if isinstance(m, str):
            m = method[m]
        self._check(lib().t1m_set_method(self._h, int(m)))

    def set_split_k(self, splits: int) -> None:
        """Force the number of K partitions (0 = automatic)."""
        self._check(lib().t1m_set_split_k(self._h, int(splits)))

    def set_workspace_limit(self, nbytes: int) -> None:
        """Cap each optional tensor-core workspace (B panels, dense operand
        packs); -1 = no cap, 0 = never use them (results are unchanged)."""
        self._check(lib().t1m_set_workspace_limit(self._h, int(nbytes)))

    def set_tile_form(self, form: int | str) -> None:
        """Tile form of tensor-core products: "auto", "one" (one tile per
        CTA) or "pair" (clusters of two CTAs sharing each MMA)."""
        if isinstance(form, str):
            form = TILE_FORMS[form]
        self._check(lib().t1m_set_tile_form(self._h, int(form)))

    def set_autotune(self, on: bool) -> None:
        """Tune single tensor-core contractions (tile form, split count) once
        per shape class; choices cached in $T1M_TUNE_CACHE."""
        self._check(lib().t1m_set_autotune(self._h, int(bool(on))))

    def set_wait_limit(self, microseconds: int) -> None:
        """Bound on grouped launches' device-side dependency waits (us; 0 =
        the default of about two seconds), for groups created afterwards."""
        self._check(lib().t1m_set_wait_limit(self._h, int(microseconds)))

    def set_stream(self, stream: int | None) -> None:
        self._check(lib().t1m_set_stream(self._h, stream or None))

    def synchronize(self) -> None:
        self._check(lib().t1m_synchronize(self._h))

    def _check(self, st: int) -> None:
        if st != OK:
            raise T1MError(st, (lib().t1m_last_error(self._h) or b"").decode())

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def close(self) -> None:
        if self._h:
            lib().t1m_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context()
    return _default_ctx


_TORCH_NP: dict | None = None


def _torch_dtypes() -> dict:
    """torch element type -> numpy dtype, built on first use (torch is
    plumbing for device memory only and need not be installed)."""
    global _TORCH_NP
    if _TORCH_NP is None:
        try:
            import torch
            _TORCH_NP = {torch.float32: np.dtype(np.float32), torch.float64: np.dtype(np.float64),
                         torch.complex64: np.dtype(np.complex64),
                         torch.complex128: np.dtype(np.complex128)}
        except ImportError:
            _TORCH_NP = {}
    return _TORCH_NP


def _data_ptr(data: Any) -> tuple[int, np.dtype]:
    if isinstance(data, np.ndarray):
        return data.ctypes.data, data.dtype
    npdt = _torch_dtypes().get(getattr(data, "dtype", None))
    if npdt is not None and hasattr(data, "data_ptr"):
        return data.data_ptr(), npdt
    raise TypeError(f"unsupported tensor storage {type(data)!r} "
                    f"(element type {getattr(data, 'dtype', None)})")


@dataclass
class tensor:
    """Non-owning tensor view, like the reference's t1m::tensor (t1m.h:31-66).

    ``data`` is a flat buffer (numpy array, torch tensor) holding the elements
    in ``layout`` order, or any array together with explicit ``strides``
    (elements)."""
    dims: Sequence[int]
    data: Any
    layout: int = col_major
    strides: Sequence[int] | None = None

    def rank(self) -> int:
        return len(self.dims)

    def dtype(self) -> np.dtype:
        return _data_ptr(self.data)[1]

    def _c(self, keep: list, ptr: int | None = None) -> _Tensor:
        if ptr is None:
            ptr = _data_ptr(self.data)[0]
        ext = (C.c_int64 * max(1, len(self.dims)))(*[int(d) for d in self.dims])
        keep.append(ext)
        t = _Tensor(len(self.dims), int(self.layout), ext, None, ptr)
        if self.strides is not None:
            st = (C.c_int64 * max(1, len(self.strides)))(*[int(s) for s in self.strides])
            keep.append(st)
            t.layout = STRIDED
            t.strides = st
        return t

    @staticmethod
    def from_array(arr: np.ndarray) -> "tensor":
        """View a numpy array with its own strides."""
        item = arr.itemsize
        return tensor(arr.shape, arr, STRIDED, [s // item for s in arr.strides])


def _scalar_bytes(dtype: int, v) -> C.Array:
    v = complex(v)
    if dtype == FLOAT32:
        return (C.c_float * 1)(v.real)
    if dtype == FLOAT64:
        return (C.c_double * 1)(v.real)
    if dtype == COMPLEX64:
        return (C.c_float * 2)(v.real, v.imag)
    return (C.c_double * 2)(v.real, v.imag)


def contract_raw(alpha, a: tensor, la: str, b: tensor, lb: str, beta, c: tensor, lc: str,
                 flags: int = 0, ctx: Context | None = None) -> Report:
    """One call of t1m_contract; returns its report."""
    (pa, da), (pb, db), (pc, dc) = _data_ptr(a.data), _data_ptr(b.data), _data_ptr(c.data)
    if not da == db == dc:
        raise TypeError(f"mixed element types {(str(da), str(db), str(dc))}")
    ctx = ctx or default_context()
    dtype = _DTYPE_OF[da]
    keep: list = []
    ta, tb, tc = a._c(keep, pa), b._c(keep, pb), c._c(keep, pc)
    al, be = _scalar_bytes(dtype, alpha), _scalar_bytes(dtype, beta)
    rep = Report()
    st = lib().t1m_contract(ctx.handle, dtype, al, C.byref(ta), la.encode(), C.byref(tb),
                            lb.encode(), be, C.byref(tc), lc.encode(), int(flags), C.byref(rep))
    if st != OK:
        raise T1MError(st, (lib().t1m_last_error(ctx.handle) or b"").decode())
    return rep


def contract(*args, ctx: Context | None = None):
    """Reference-compatible contraction (t1m.h:560-577), C <- C + alpha*A*B.

    ``contract(a, la, b, lb, c, lc)`` for complex tensors;
    ``contract(alpha, a, la, b, lb, beta, c, lc)`` for real tensors (beta is
    accepted and ignored, as in the reference)."""
    if len(args) == 6:
        a, la, b, lb, c, lc = args
        if a.dtype().kind != "c":
            raise TypeError("the 6-argument overload is for complex tensors (t1m.h:570-577)")
        return contract_raw(1.0, a, la, b, lb, 0.0, c, lc, FLAG_ACCUMULATE, ctx)
    if len(args) == 8:
        alpha, a, la, b, lb, beta, c, lc = args
        if a.dtype().kind == "c":
            raise TypeError("the 8-argument overload is for real tensors (t1m.h:560-568)")
        return contract_raw(alpha, a, la, b, lb, beta, c, lc, FLAG_ACCUMULATE, ctx)
    raise TypeError("contract takes 6 (complex) or 8 (real) positional arguments")


def contract_scaled(alpha, a: tensor, la: str, b: tensor, lb: str, beta, c: tensor, lc: str,
                    ctx: Context | None = None, conj_a: bool = False,
                    conj_b: bool = False) -> Report:
    """C <- alpha*op(A)*op(B) + beta*C with complex alpha/beta (no reference
    counterpart; the reference has no complex scalars, t1m.h:570-577)."""
    flags = (FLAG_CONJ_A if conj_a else 0) | (FLAG_CONJ_B if conj_b else 0)
    return contract_raw(alpha, a, la, b, lb, beta, c, lc, flags, ctx)


def contract_vjp(dc: tensor, lc: str, a: tensor, la: str, b: tensor, lb: str,
                 da: tensor | None = None, db: tensor | None = None,
                 accumulate: bool = False, ctx: Context | None = None,
                 timed: bool = True) -> Report:
    """Adjoint of C = A*B: dA = dC*conj(B), dB = conj(A)*dC (conjugate-Wirtinger
    convention of PyTorch's complex autograd).  da/db may be None.  With
    timed=False the calls stay asynchronous on the context's stream (no
    per-call events or synchronisation; the report carries no times)."""
    ctx = ctx or default_context()
    dts = {dc.dtype(), a.dtype(), b.dtype()}
    if len(dts) != 1:
        raise TypeError(f"mixed element types {dts}")
    dtype = _DTYPE_OF[dts.pop()]
    keep: list = []
    tdc, ta, tb = dc._c(keep), a._c(keep), b._c(keep)
    pda = C.byref(da._c(keep)) if da is not None else None
    pdb = C.byref(db._c(keep)) if db is not None else None
    rep = Report()
    st = lib().t1m_contract_vjp(ctx.handle, dtype, C.byref(tdc), lc.encode(), C.byref(ta),
                                la.encode(), C.byref(tb), lb.encode(), pda, pdb,
                                (FLAG_ACCUMULATE if accumulate else 0) |
                                (0 if timed else FLAG_NO_TIMING), C.byref(rep))
    if st != OK:
        raise T1MError(st, (lib().t1m_last_error(ctx.handle) or b"").decode())
    return rep


class Group:
    """A batch of contractions run as grouped launches (t1m_group_*).

    ``items``: sequence of (alpha, a, la, b, lb, beta, c, lc, depends_on
    [, flags]) with device tensors (C = alpha*A*B + beta*C; depends_on =
    index of an earlier item whose C this one reads, or -1; flags: FLAG_CONJ_A
    / FLAG_CONJ_B / FLAG_ACCUMULATE, default 0)."""

    def __init__(self, items, ctx: Context | None = None, graph: bool = True,
                 autotune: bool = False, options: int = 0):
        self.ctx = ctx or default_context()
        self._h = C.c_void_p()
        self._keep: list = []
        arr = (GroupItem * max(1, len(items)))()
        dtypes = set()
        for i, item in enumerate(items):
            alpha, a, la, b, lb, beta, c, lc, dep = item[:9]
            flags = int(item[9]) if len(item) > 9 else 0
            dtypes |= {a.dtype(), b.dtype(), c.dtype()}
            ta, tb, tc = a._c(self._keep), b._c(self._keep), c._c(self._keep)
            self._keep += [ta, tb, tc]
            al, be = complex(alpha), complex(beta)
            arr[i] = GroupItem(C.pointer(ta), la.encode(), C.pointer(tb), lb.encode(),
                               C.pointer(tc), lc.encode(), (C.c_double * 2)(al.real, al.imag),
                               (C.c_double * 2)(be.real, be.imag), int(dep), flags)
        if len(dtypes) > 1:
            raise TypeError(f"mixed element types {dtypes}")
        dtype = _DTYPE_OF[dtypes.pop()] if dtypes else COMPLEX64
        self._keep.append(arr)
        opts = (GROUP_GRAPH if graph else 0) | (GROUP_AUTOTUNE if autotune else 0) | options
        st = lib().t1m_group_create(self.ctx.handle, dtype, len(items), arr, opts,
                                    C.byref(self._h))
        if st != OK:
            raise T1MError(st, (lib().t1m_last_error(self.ctx.handle) or b"").decode())

    def launch(self, timed: bool = True) -> Report | None:
        rep = Report()
        st = lib().t1m_group_launch(self._h, C.byref(rep) if timed else None)
        if st != OK:
            raise T1MError(st, (lib().t1m_last_error(self.ctx.handle) or b"").decode())
        return rep if timed else None

    def close(self) -> None:
        if self._h:
            lib().t1m_group_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def analyze(a: tensor, la: str, b: tensor, lb: str, c: tensor, lc: str) -> dict:
    """Label analysis only (no GPU): matricised M, N, K or a T1MError."""
    dts = {a.dtype(), b.dtype(), c.dtype()}
    dtype = _DTYPE_OF[dts.pop()] if len(dts) == 1 else -1
    keep: list = []
    ta, tb, tc = a._c(keep), b._c(keep), c._c(keep)
    info = PlanInfo()
    err = C.create_string_buffer(512)
    st = lib().t1m_analyze(dtype, C.byref(ta), la.encode(), C.byref(tb), lb.encode(),
                           C.byref(tc), lc.encode(), C.byref(info), err, 512)
    if st != OK:
        raise T1MError(st, err.value.decode())
    return {"m": info.m, "n": info.n, "k": info.k, "modes": (info.modes_m, info.modes_n,
                                                              info.modes_k)}


def version() -> tuple[int, int, int]:
    ma, mi, sm = C.c_int(), C.c_int(), C.c_int()
    lib().t1m_version(C.byref(ma), C.byref(mi), C.byref(sm))
    return ma.value, mi.value, sm.value
