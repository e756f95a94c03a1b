"""The profiled FP32 pressure-gradient entry points without a GPU: argument checks.

oeb_p_grad_c_f32_profiled / oeb_nh_p_grad_f32_profiled check their descriptors exactly as
the standard FP32 entry points do, then their base-profile pointers, all before any CUDA call;
these calls return at one of those checks, so nothing is launched or dereferenced.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

H = 3
PROFILED = {"p_grad_c": 2, "nh_p_grad": 3}  # base profiles each entry point takes


def _call(pkg, fields, name, bases, halo=H, nx=8, ny=8, nz=2):
    spec = pkg.KERNELS[name]
    inputs = fields.make_inputs(name, nx, ny, nz, seed=1, halo=halo)
    outs = fields.make_outputs(name, nx, ny, nz, halo=halo)
    st = {k: pkg.Storage(v.astype(np.float32), halo) for k, v in {**inputs, **outs}.items()}
    args = [ctypes.byref(st[a.name].memref()) for a in spec.abi_args]
    scal = [ctypes.c_float(0.05) for _ in spec.scalars]
    dom = pkg.Domain(nx, ny, nz)
    fn = getattr(pkg.load_library(), "oeb_%s_f32_profiled" % name)
    fn.restype = ctypes.c_int
    return fn(*args, *bases, *scal, ctypes.byref(dom), ctypes.c_void_p(0))


@pytest.mark.parametrize("name", sorted(PROFILED))
def test_null_base_profile_is_rejected(pkg, fields, name):
    host = np.zeros(3)  # never read: the call returns at the NULL check
    for hole in range(PROFILED[name]):
        bases = [ctypes.c_void_p(0 if q == hole else host.ctypes.data) for q in range(PROFILED[name])]
        assert _call(pkg, fields, name, bases) == 1  # OEB_ERR_NULL


@pytest.mark.parametrize("name", sorted(PROFILED))
def test_descriptors_are_checked_before_the_profiles(pkg, fields, name):
    need = pkg.KERNELS[name].max_halo
    bases = [ctypes.c_void_p(0)] * PROFILED[name]
    assert _call(pkg, fields, name, bases, halo=need - 1) == 4  # OEB_ERR_HALO, not OEB_ERR_NULL


def test_python_wrapper_checks_its_arguments(pkg, fields):
    inputs = fields.make_inputs("p_grad_c", 8, 8, 2, seed=1)
    outs = fields.make_outputs("p_grad_c", 8, 8, 2)
    st = {k: pkg.Storage(v.astype(np.float32), H) for k, v in {**inputs, **outs}.items()}
    with pytest.raises(ValueError, match="no profiled form"):
        pkg.kernels.call_profiled("laplace", st, {}, domain=(8, 8, 2))
    with pytest.raises(TypeError, match="FP32 device Storages"):
        pkg.kernels.call_profiled("p_grad_c", st, {}, domain=(8, 8, 2))
    assert pkg.kernels.PROFILED_FIELDS == {"p_grad_c": ("gz", "pkc"), "nh_p_grad": ("gz", "pp", "pk3")}
