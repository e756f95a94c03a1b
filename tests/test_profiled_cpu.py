"""The profiled FP32 pressure-gradient entry points without a GPU.

* Argument checks: oeb_p_grad_c_f32_profiled / oeb_nh_p_grad_f32_profiled check their
  descriptors exactly as the standard FP32 entry points do, then their base-profile pointers,
  all before any CUDA call; these calls return at one of those checks, so nothing is launched
  or dereferenced.
* The storage format's own error floor, through the FP64 oracle.
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


@pytest.mark.parametrize("name", sorted(PROFILED))
@pytest.mark.parametrize("case", [("fronts", 37, 45, 5, 9), ("physical", 64, 48, 20, 1)])
def test_profiled_storage_floor(pkg, fields, orc, name, case):
    """The storage format alone, through the FP64 oracle: outputs from the fields as an FP64
    per-level base plus FP32 perturbations are within 1e-6 of those from the FP64 fields (the
    floor the GPU kernels' total error sits on), while full-value FP32 fields are not."""
    workload, nx, ny, nz, seed = case
    spec = pkg.KERNELS[name]
    inputs = fields.make_inputs(name, nx, ny, nz, seed=seed, workload=workload)
    outs = fields.make_outputs(name, nx, ny, nz)
    sc = fields.make_scalars(name, seed=seed)
    ref = {k: v.copy() for k, v in {**inputs, **outs}.items()}
    orc.run_oracle(spec, ref, sc, nx, ny, nz, H)
    prof = {k: v.copy() for k, v in {**inputs, **outs}.items()}
    full = {k: v.copy() for k, v in {**inputs, **outs}.items()}
    for f in pkg.kernels.PROFILED_FIELDS[name]:
        a = inputs[f]
        base = a[H:H + nz + 1].mean(axis=(1, 2))
        pert = (a[H:H + nz + 1] - base[:, None, None]).astype(np.float32)
        prof[f][H:H + nz + 1] = base[:, None, None] + pert.astype(np.float64)
        full[f] = a.astype(np.float32).astype(np.float64)
    orc.run_oracle(spec, prof, sc, nx, ny, nz, H)
    orc.run_oracle(spec, full, sc, nx, ny, nz, H)
    box = (slice(H, H + nz), slice(H, H + ny), slice(H, H + nx))
    for a in spec.by_role("out3"):
        want = ref[a.name][box]
        scale = np.abs(want).max()
        e_prof = np.abs(prof[a.name][box] - want).max() / scale
        e_full = np.abs(full[a.name][box] - want).max() / scale
        assert e_prof <= 3e-7, (name, a.name, e_prof)
        assert e_full > 1e-6, (name, a.name, e_full)
