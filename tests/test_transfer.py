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
