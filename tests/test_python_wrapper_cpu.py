"""The Python mirror's argument handling (no GPU): storage pointers and element
types of numpy and torch operands, the ctypes tensor descriptors, and the
errors raised before any device work."""
import ctypes as C

import numpy as np
import pytest

import t1m_gb300 as t1m


def test_numpy_storage_pointer_and_type():
    a = np.zeros((3, 4), np.complex64)
    ptr, dt = t1m._data_ptr(a)
    assert ptr == a.ctypes.data and dt == np.dtype(np.complex64)


def test_torch_storage_pointer_and_type():
    torch = pytest.importorskip("torch")
    for tdt, ndt in ((torch.float32, np.float32), (torch.float64, np.float64),
                     (torch.complex64, np.complex64), (torch.complex128, np.complex128)):
        x = torch.zeros(5, dtype=tdt)
        ptr, dt = t1m._data_ptr(x)
        assert ptr == x.data_ptr() and dt == np.dtype(ndt)


def test_unsupported_storage_is_a_type_error():
    torch = pytest.importorskip("torch")
    with pytest.raises(TypeError, match="float16"):
        t1m._data_ptr(torch.zeros(2, dtype=torch.float16))
    with pytest.raises(TypeError):
        t1m._data_ptr([1.0, 2.0])


def test_descriptor_fields():
    a = np.zeros((2, 3, 4), np.float64)
    keep = []
    d = t1m.tensor([2, 3, 4], a, t1m.row_major)._c(keep)
    assert d.ndim == 3 and d.layout == int(t1m.row_major) and d.data == a.ctypes.data
    assert [d.extents[i] for i in range(3)] == [2, 3, 4] and not d.strides
    # Explicit strides switch the descriptor to the strided layout; an explicit
    # pointer (the caller already looked it up) is used as given.
    s = t1m.tensor([2, 3], a, t1m.col_major, [12, 4])._c(keep, 12345)
    assert s.layout == t1m.STRIDED and [s.strides[i] for i in range(2)] == [12, 4]
    assert s.data == 12345


def test_from_array_uses_element_strides():
    a = np.zeros((4, 6), np.complex64)[:, ::2]
    t = t1m.tensor.from_array(a)
    assert list(t.dims) == [4, 3] and list(t.strides) == [6, 2] and t.layout == t1m.STRIDED


def test_mixed_element_types_fail_before_any_device_work():
    a = np.zeros((2, 2), np.complex64)
    b = np.zeros((2, 2), np.complex128)
    with pytest.raises(TypeError, match="mixed element types"):
        t1m.contract_raw(1.0, t1m.tensor([2, 2], a), "ab", t1m.tensor([2, 2], b), "bc", 0.0,
                         t1m.tensor([2, 2], a), "ac")


def test_scalar_encoding():
    assert list(t1m._scalar_bytes(t1m.COMPLEX64, 1 - 2j)) == [1.0, -2.0]
    assert list(t1m._scalar_bytes(t1m.FLOAT64, 3.5)) == [3.5]
    assert C.sizeof(t1m._scalar_bytes(t1m.COMPLEX128, 1j)) == 16


def test_constants_mirror_the_c_header():
    """Every T1M_FLAG_*, T1M_GROUP_* and T1M_PATH_* flag of include/t1m_capi.h
    has the same value in the Python mirror (GROUP_*, FLAG_*, PATH_*), and the
    tile forms match T1M_TILE_*."""
    import re
    from pathlib import Path

    import t1m_gb300 as t1m
    hdr = (Path(__file__).resolve().parents[1] / "include" / "t1m_capi.h").read_text()
    defs = {m.group(1): int(m.group(2), 0)
            for m in re.finditer(r"^#define T1M_(\w+) (0x[0-9A-Fa-f]+|\d+)u?\b", hdr, re.M)}
    checked = 0
    for name, value in defs.items():
        if name.startswith(("FLAG_", "GROUP_", "PATH_")) and name != "PATH_B_PANELS":
            assert getattr(t1m, name) == value, name
            checked += 1
        elif name.startswith("TILE_"):
            assert t1m.TILE_FORMS[name[5:].lower()] == value, name
            checked += 1
    assert checked >= 20, checked
