"""numpy restatement of the reference's hot path + the FP64 oracle.

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` as the checker, never by the product.

Each function restates one piece of include/t1m/t1m.h (cited per function) so
that the golden vectors of the reference's own unit tests
(test/test_scatter.cpp, test/test_packing.cpp) can be checked against it, and
so that GPU results can be compared with an exact-arithmetic-grade FP64
result.
"""
from __future__ import annotations

import numpy as np


# ---------------------------------------------------------------- layouts ---
def col_major_strides(dims):
    """Column-major element strides, t1m.h:45-50 (s0 = 1, si = s(i-1)*d(i-1))."""
    s, acc = [], 1
    for d in dims:
        s.append(acc)
        acc *= int(d)
    return s


def row_major_strides(dims):
    """Row-major element strides (the reference leaves these unset, t1m.h:51-52;
    here the last mode is unit stride)."""
    s, acc = [0] * len(dims), 1
    for i in range(len(dims) - 1, -1, -1):
        s[i] = acc
        acc *= int(dims[i])
    return s


# ---------------------------------------------------------------- bundles ---
def index_bundles(la: str, lb: str, lc: str):
    """Restates get_index_bundles, t1m.h:90-136.

    contracted = sorted(A & B), free_a = sorted(A - B), free_b = sorted(B - A);
    A.X = free_a in A, A.Y = contracted in A, B.X = contracted in B,
    B.Y = free_b in B, C.X = free_a in C, C.Y = free_b in C.
    """
    sa, sb = set(la), set(lb)
    contracted = sorted(sa & sb)
    free_a = sorted(sa - sb)
    free_b = sorted(sb - sa)
    return {
        "AX": [la.find(ch) for ch in free_a],
        "AY": [la.find(ch) for ch in contracted],
        "BX": [lb.find(ch) for ch in contracted],
        "BY": [lb.find(ch) for ch in free_b],
        "CX": [lc.find(ch) for ch in free_a],
        "CY": [lc.find(ch) for ch in free_b],
    }


def scatter(indices, dims, strides) -> np.ndarray:
    """Restates get_scatter, t1m.h:141-174: offsets of every element of the
    bundle, first listed mode fastest."""
    out = np.zeros(1, dtype=np.int64)
    for idx in reversed(list(indices)):
        part = np.arange(int(dims[idx]), dtype=np.int64) * int(strides[idx])
        out = (out[:, None] + part[None, :]).reshape(-1)
    return out


def block_scatter(scat, b: int) -> np.ndarray:
    """Restates get_block_scatter, t1m.h:179-205: per block of ``b`` entries the
    constant stride, or 0 when the block is not uniform or has one entry."""
    scat = np.asarray(scat, dtype=np.int64)
    out = []
    for i in range(0, len(scat), b):
        blk = scat[i:i + b]
        if len(blk) == 1:
            out.append(0)
            continue
        d = np.diff(blk)
        out.append(int(d[-1]) if np.all(d == d[0]) else 0)
    return np.asarray(out, dtype=np.int64)


# ---------------------------------------------------------------- packing ---
def _matrix(dims, bundle_x, bundle_y, strides=None):
    strides = col_major_strides(dims) if strides is None else strides
    return scatter(bundle_x, dims, strides), scatter(bundle_y, dims, strides)


def pack_block(src, dims, bx, by, br, bc, length, label, complex_1m, dest_len):
    """Restates pack_block/pack_cell, t1m.h:279-404 (column-major tensor).

    label "A": MR-tall column-major slivers; "B": NR-wide row-major slivers.
    complex_1m: A cells become [re -im; im re], B rows become re/im pairs.
    Returns the packed real buffer (zero padded, like the reference's zeroed
    workspace)."""
    src = np.asarray(src).reshape(-1)
    rs, cs = _matrix(dims, bx, by)
    real_t = np.float32 if src.dtype in (np.float32, np.complex64) else np.float64
    dest = np.zeros(dest_len, dtype=real_t)
    for row in range(len(rs)):
        for col in range(len(cs)):
            v = src[rs[row] + cs[col]]
            if not complex_1m:
                if label == "A":
                    dest[(row // br) * br * length + col * br + row % br] = v
                else:
                    dest[(col // bc) * bc * length + row * bc + col % bc] = v
            else:
                if label == "A":
                    hb = br // 2
                    base = 2 * col * br + 2 * (row // hb) * hb * length + 2 * (row % hb)
                    dest[base] = v.real
                    dest[base + 1] = v.imag
                    dest[base + br] = -v.imag
                    dest[base + br + 1] = v.real
                else:
                    base = 2 * row * bc + (col // bc) * bc * length + col % bc
                    dest[base] = v.real
                    dest[base + bc] = v.imag
    return dest


def unpack(src, dims, bx, by, br, dest, complex_1m):
    """Restates unpack, t1m.h:406-430: scatter-ADD a packed tile into dest."""
    rs, cs = _matrix(dims, bx, by)
    src = np.asarray(src).reshape(-1)
    dest = np.array(dest, copy=True).reshape(-1)
    for l in range(len(cs)):
        for k in range(len(rs)):
            if complex_1m:
                si = 2 * k + l * br
                dest[rs[k] + cs[l]] += src[si] + 1j * src[si + 1]
            else:
                dest[rs[k] + cs[l]] += src[k + l * br]
    return dest


# ------------------------------------------------------------ FP64 oracle ---
def einsum_spec(la: str, lb: str, lc: str) -> str:
    return f"{la},{lb}->{lc}"


def as_strided_view(flat: np.ndarray, dims, strides) -> np.ndarray:
    """View a flat element buffer as a tensor with the given element strides."""
    item = flat.dtype.itemsize
    return np.lib.stride_tricks.as_strided(
        flat, shape=tuple(int(d) for d in dims),
        strides=tuple(int(s) * item for s in strides))


def contract_fp64(a, la, b, lb, c0, lc, alpha=1.0, beta=0.0, accumulate=False):
    """FP64 (complex128 / float64) result of the contraction.

    ``a``, ``b``, ``c0`` are numpy tensors in logical index order (any
    strides).  accumulate=True gives the reference's semantics
    C0 + alpha*A*B (beta ignored, t1m.h:497-502, 543-548); otherwise BLAS
    semantics alpha*A*B + beta*C0.
    """
    wide = np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64
    ab = np.einsum(einsum_spec(la, lb, lc), a.astype(wide), b.astype(wide),
                   optimize=True)
    if accumulate:
        return c0.astype(wide) + alpha * ab
    out = alpha * ab
    if beta != 0:
        out = out + beta * c0.astype(wide)
    return out


def matricize(la, lb, lc, dims_a, dims_b, dims_c, sa, sb, sc):
    """Scatter vectors (rsA, csA, rsB, csB, rsC, csC) of the three operands in
    the reference's bundle order."""
    bd = index_bundles(la, lb, lc)
    return (scatter(bd["AX"], dims_a, sa), scatter(bd["AY"], dims_a, sa),
            scatter(bd["BX"], dims_b, sb), scatter(bd["BY"], dims_b, sb),
            scatter(bd["CX"], dims_c, sc), scatter(bd["CY"], dims_c, sc))


def sampled_entries(flat_a, flat_b, scat, rows, cols):
    """FP64 values of C = A*B at the sampled matricised (row, col) pairs.

    Used at sizes where a full FP64 contraction is too slow: each sample is one
    K-long dot product in complex128."""
    rsA, csA, rsB, csB = scat[:4]
    wide = np.complex128 if np.iscomplexobj(flat_a) else np.float64
    out = np.empty(len(rows), dtype=wide)
    chunk = 256
    for s in range(0, len(rows), chunk):
        r = rows[s:s + chunk]
        c = cols[s:s + chunk]
        av = flat_a[rsA[r][:, None] + csA[None, :]].astype(wide)   # (S, K)
        bv = flat_b[rsB[None, :] + csB[c][:, None]].astype(wide)   # (S, K)
        out[s:s + chunk] = np.einsum("sk,sk->s", av, bv)
    return out


def rel_errors(got, ref):
    """(normwise max, Frobenius) relative error of ``got`` against ``ref``."""
    ref = np.asarray(ref)
    cplx = np.iscomplexobj(ref) or np.iscomplexobj(got)
    got = np.asarray(got).astype(np.complex128 if cplx else np.float64)
    d = np.abs(got - ref)
    mx = float(d.max() / max(np.abs(ref).max(), np.finfo(np.float64).tiny))
    fro = float(np.linalg.norm(d.reshape(-1)) /
                max(np.linalg.norm(ref.reshape(-1)), np.finfo(np.float64).tiny))
    return mx, fro
