"""oeb_upload* / oeb_download*: a field made in host memory moves to its device twin and back.

A transfer copies the descriptor's whole span (halo and row padding included), so a round
trip must return every cell bit for bit.  Descriptors of different layouts, NULL ones and
overlapping spans are refused with their status before any CUDA call, which the CPU tests
check.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import assert_bitwise_equal

H = 3
OEB_ERR_NULL, OEB_ERR_LAYOUT, OEB_ERR_ALIAS = 1, 3, 8


def _fn(pkg, name):
    fn = getattr(pkg.load_library(), name)
    fn.restype = ctypes.c_int
    return fn


def _ref(st):
    return ctypes.byref(st.memref())


def _field(shape, dtype, seed):
    return np.random.default_rng(seed).standard_normal(shape).astype(dtype)


@pytest.mark.parametrize("p", ["f64", "f32"])
def test_transfers_refuse_bad_descriptors_before_any_cuda_call(pkg, p):
    dt = np.float64 if p == "f64" else np.float32
    a = pkg.Storage(_field((5 + 2 * H, 4 + 2 * H, 6 + 2 * H), dt, 1), H)
    b = pkg.Storage(_field((5 + 2 * H, 4 + 2 * H, 7 + 2 * H), dt, 2), H)  # one column wider
    c = pkg.Storage(_field((5 + 2 * H, 4 + 2 * H, 6 + 2 * H), dt, 3), H - 1)  # another offset
    for name in ("oeb_upload3d_" + p, "oeb_download3d_" + p):
        fn = _fn(pkg, name)
        assert fn(None, _ref(a), None) == OEB_ERR_NULL
        assert fn(_ref(a), None, None) == OEB_ERR_NULL
        assert fn(_ref(a), _ref(b), None) == OEB_ERR_LAYOUT
        assert fn(_ref(a), _ref(c), None) == OEB_ERR_LAYOUT
        assert fn(_ref(a), _ref(a), None) == OEB_ERR_ALIAS
    u = pkg.Storage(_field((9 + 2 * H,), dt, 4), H)
    v = pkg.Storage(_field((8 + 2 * H,), dt, 5), H)
    for name in ("oeb_upload1d_" + p, "oeb_download1d_" + p):
        fn = _fn(pkg, name)
        assert fn(None, _ref(u), None) == OEB_ERR_NULL
        assert fn(_ref(u), _ref(v), None) == OEB_ERR_LAYOUT
        assert fn(_ref(u), _ref(u), None) == OEB_ERR_ALIAS


@pytest.mark.gpu
@pytest.mark.parametrize("p", ["f64", "f32"])
def test_upload_then_download_returns_every_cell(pkg, cuda, p):
    import torch
    dt = np.float64 if p == "f64" else np.float32
    tdt = torch.float64 if p == "f64" else torch.float32
    stream = torch.cuda.current_stream(cuda)
    for shape, up, down in (((9 + 2 * H, 7 + 2 * H, 11 + 2 * H), "oeb_upload3d_", "oeb_download3d_"),
                            ((13 + 2 * H,), "oeb_upload1d_", "oeb_download1d_")):
        a = _field(shape, dt, 7)
        host = pkg.Storage(a.copy(), H)
        dev = pkg.Storage(torch.zeros(shape, dtype=tdt, device=cuda), H)
        assert _fn(pkg, up + p)(_ref(dev), _ref(host), ctypes.c_void_p(stream.cuda_stream)) == 0
        torch.cuda.synchronize()
        assert_bitwise_equal(dev.data.cpu().numpy(), a, "%s%s" % (up, p))
        dev.data.mul_(-2.0)
        back = pkg.Storage(np.zeros_like(a), H)
        assert _fn(pkg, down + p)(_ref(back), _ref(dev), ctypes.c_void_p(stream.cuda_stream)) == 0
        torch.cuda.synchronize()
        assert_bitwise_equal(back.data, -2.0 * a, "%s%s" % (down, p))


def _util_h_layout(a: np.ndarray, halo: int, rank: int):
    """A host descriptor as the reference's allocateStorage makes it (include/util.h:99-141):
    aligned = allocated + (32 - halo), the elements starting at aligned[0]."""
    pad = 32 - halo
    buf = np.zeros(pad + a.size, dtype=a.dtype)
    buf[pad:] = a.ravel()
    base = buf.ctypes.data
    aligned = base + pad * a.itemsize
    if rank == 3:
        szk, szj, szi = a.shape
        m = pkg_storage().Memref3d(base, aligned, halo * szj * szi + halo * szi + halo, (szk, szj, szi),
                                   (szj * szi, szi, 1))
    else:
        m = pkg_storage().Memref1d(base, aligned, halo, (a.shape[0],), (1,))
    return buf, m


def pkg_storage():
    import importlib
    return importlib.import_module("oeb_gb300.storage")


@pytest.mark.parametrize("p", ["f64", "f32"])
def test_allocate_storage_layout_pairs_with_a_twin_of_aligned_equal_allocated(pkg, p):
    # allocateStorage puts aligned 32 - halo elements above allocated; the device allocator puts
    # it at allocated.  The pair must not be refused as a layout mismatch (a CUDA error is the
    # only other answer on a machine without a GPU).
    dt = np.float64 if p == "f64" else np.float32
    a = _field((5 + 2 * H, 4 + 2 * H, 6 + 2 * H), dt, 21)
    keep, host = _util_h_layout(a, H, 3)
    twin = pkg.Storage(np.zeros_like(a), H)
    for name, args in (("oeb_upload3d_" + p, (ctypes.byref(twin.memref()), ctypes.byref(host))),
                       ("oeb_download3d_" + p, (ctypes.byref(host), ctypes.byref(twin.memref())))):
        st = _fn(pkg, name)(*args, None)
        assert st in (0, 6), "%s refused an allocateStorage-layout field: status %d" % (name, st)
    u = _field((9 + 2 * H,), dt, 22)
    keep1, host1 = _util_h_layout(u, H, 1)
    twin1 = pkg.Storage(np.zeros_like(u), H)
    st = _fn(pkg, "oeb_upload1d_" + p)(ctypes.byref(twin1.memref()), ctypes.byref(host1), None)
    assert st in (0, 6)


@pytest.mark.gpu
@pytest.mark.parametrize("p", ["f64", "f32"])
def test_allocate_storage_field_round_trips_through_its_device_twin(pkg, cuda, p):
    # host: allocateStorage's layout; device: oeb_storage3d_alloc_<p> of the same sizes and halo
    import torch
    dt = np.float64 if p == "f64" else np.float32
    nx, ny, nz = 11, 9, 7
    a = _field((nz + 2 * H, ny + 2 * H, nx + 2 * H), dt, 23)
    keep, host = _util_h_layout(a, H, 3)
    st_mod = pkg_storage()
    dev = st_mod.Memref3d()
    lib = pkg.load_library()
    assert _fn(pkg, "oeb_storage3d_alloc_" + p)(ctypes.c_int64(nx), ctypes.c_int64(ny), ctypes.c_int64(nz),
                                                 ctypes.c_int64(H), ctypes.c_int64(1), ctypes.byref(dev)) == 0
    try:
        stream = ctypes.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
        assert _fn(pkg, "oeb_upload3d_" + p)(ctypes.byref(dev), ctypes.byref(host), stream) == 0
        keep[:] = 0
        assert _fn(pkg, "oeb_download3d_" + p)(ctypes.byref(host), ctypes.byref(dev), stream) == 0
        torch.cuda.synchronize()
        assert_bitwise_equal(keep[32 - H:].reshape(a.shape), a, "allocateStorage layout round trip %s" % p)
        assert not np.any(keep[:32 - H]), "the padding before aligned was written"
    finally:
        lib.oeb_storage_free(ctypes.byref(dev))
