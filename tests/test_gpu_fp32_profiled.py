"""FP32 p_grad_c / nh_p_grad on profile-relative fields, on the GPU, through the C ABI.

The pressure, geopotential and Exner fields of these two stencils are a per-level profile
(about 1000, falling by about 11 a level) plus a 1 % horizontal perturbation.  Stored in FP32
as full values their rounding dominates the outputs' error (normwise 0.9-2.3e-5, the
``total`` column of test_gpu_fp32).  oeb_p_grad_c_f32_profiled / oeb_nh_p_grad_f32_profiled
take those fields as FP32 perturbations from an FP64 per-level base profile (here: the mean of
each level), so only the perturbations are rounded.  Checked here:

* ``total`` against the FP64 oracle on the original FP64 fields: at most 1e-6 normwise;
* ``arith`` against the FP64 oracle on the fields the kernel is given exactly
  (base + the FP32 perturbation, in FP64): at most 1e-6;
* with zero base profiles the profiled form computes bit for bit what the standard FP32 entry
  point does on the same (full-value) fields;
* a NULL base profile is OEB_ERR_NULL.
"""
from __future__ import annotations

import ctypes
import json
import os
from pathlib import Path

import numpy as np
import pytest

from conftest import assert_bitwise_equal

pytestmark = pytest.mark.gpu

H = 3
TOL = 1e-6
OEB_ERR_NULL = 1  # include/oeb_gb300.h
CASES = [("fronts", 256, 256, 80, 2), ("physical", 128, 128, 80, 1), ("fronts", 37, 45, 5, 9)]
NAMES = ("p_grad_c", "nh_p_grad")
# the measured errors are also written, as JSON, to the file OEB_FP32_PROFILED_REPORT names (if set)
REPORT = Path(os.environ["OEB_FP32_PROFILED_REPORT"]) if os.environ.get("OEB_FP32_PROFILED_REPORT") else None
_results = {}


def _box(arr, reach, nx, ny, nz, h=H):
    ilo, ihi, jlo, jhi, klo, khi = reach
    return arr[h - klo:h + nz + khi, h - jlo:h + ny + jhi, h - ilo:h + nx + ihi]


def _split(arr, nz):
    """(base, perturbation): base[k] the mean of interior level k = 0 .. nz (the levels the
    stencils read), the perturbation arr - base rounded to FP32 on those levels (the other
    levels are not read; they keep the full value)."""
    base = arr[H:H + nz + 1].mean(axis=(1, 2))
    pert = arr.copy()
    pert[H:H + nz + 1] -= base[:, None, None]
    return base, pert.astype(np.float32)


def _setup(pkg, fields, name, nx, ny, nz, seed, workload):
    spec = pkg.KERNELS[name]
    inputs = fields.make_inputs(name, nx, ny, nz, seed=seed, workload=workload)
    sc = fields.make_scalars(name, seed=seed)
    outs = fields.make_outputs(name, nx, ny, nz)
    sc32 = {s.name: (sc[s.name] if s.always_double else float(np.float32(sc[s.name]))) for s in spec.scalars}
    return spec, inputs, outs, sc, sc32


def _run_profiled(pkg, cuda, name, spec, inputs, outs, bases, perts, sc32, nx, ny, nz):
    import torch
    host = {k: v.astype(np.float32) for k, v in {**inputs, **outs}.items()}
    host.update(perts)
    dev = {k: pkg.Storage(torch.from_numpy(v).to(cuda), H) for k, v in host.items()}
    db = {k: torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)).to(cuda) for k, b in bases.items()}
    pkg.kernels.call_profiled(name, dev, db, sc32, domain=(nx, ny, nz))
    torch.cuda.synchronize()
    return dev


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("case", CASES)
def test_profiled_error_vs_fp64_oracle(pkg, fields, orc, cuda, name, case):
    workload, nx, ny, nz, seed = case
    spec, inputs, outs, sc, sc32 = _setup(pkg, fields, name, nx, ny, nz, seed, workload)
    bases, perts = {}, {}
    for f in pkg.kernels.PROFILED_FIELDS[name]:
        bases[f], perts[f] = _split(inputs[f], nz)
    # the FP64 oracle on the original fields, and on the fields the kernel is given exactly
    ref = {k: v.copy() for k, v in {**inputs, **outs}.items()}
    orc.run_oracle(spec, ref, sc, nx, ny, nz, H)
    given = {k: v.astype(np.float32).astype(np.float64) for k, v in {**inputs, **outs}.items()}
    for f in bases:
        g = inputs[f].astype(np.float32).astype(np.float64)
        g[H:H + nz + 1] = bases[f][:, None, None] + perts[f][H:H + nz + 1].astype(np.float64)
        given[f] = g
    orc.run_oracle(spec, given, sc32, nx, ny, nz, H)
    dev = _run_profiled(pkg, cuda, name, spec, inputs, outs, bases, perts, sc32, nx, ny, nz)
    for a in spec.by_role("out3"):
        want = _box(ref[a.name], a.reach, nx, ny, nz)
        want_g = _box(given[a.name], a.reach, nx, ny, nz)
        got = _box(dev[a.name].numpy(), a.reach, nx, ny, nz).astype(np.float64)
        scale = np.abs(want).max()
        e_tot = float(np.abs(got - want).max() / scale)
        e_ar = float(np.abs(got - want_g).max() / scale)
        what = "%s.%s %s" % (name, a.name, case)
        _results["%s.%s/%s_%dx%dx%d" % (name, a.name, workload, nx, ny, nz)] = {"total_max": e_tot, "arith_max": e_ar}
        if REPORT is not None:
            REPORT.parent.mkdir(parents=True, exist_ok=True)
            REPORT.write_text(json.dumps(_results, indent=1, sort_keys=True))
        assert e_ar <= TOL, "%s: arithmetic error %.3g" % (what, e_ar)
        assert e_tot <= TOL, "%s: total error %.3g" % (what, e_tot)
        # cells outside the written box keep their value
        full = dev[a.name].numpy()
        mask = np.ones_like(full, dtype=bool)
        ilo, ihi, jlo, jhi, klo, khi = a.reach
        mask[H - klo:H + nz + khi, H - jlo:H + ny + jhi, H - ilo:H + nx + ihi] = False
        assert (full[mask] == np.float32(fields.SENTINEL)).all(), "%s wrote outside its box" % what


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("size", [(128, 128, 80), (37, 45, 5)], ids=["128x128x80", "37x45x5"])
def test_zero_profile_is_the_standard_entry(pkg, fields, cuda, name, size):
    import torch
    nx, ny, nz = size
    spec, inputs, outs, sc, sc32 = _setup(pkg, fields, name, nx, ny, nz, 4, "fronts")
    zero = {f: np.zeros(nz + 1) for f in pkg.kernels.PROFILED_FIELDS[name]}
    perts = {f: inputs[f].astype(np.float32) for f in zero}
    dev = _run_profiled(pkg, cuda, name, spec, inputs, outs, zero, perts, sc32, nx, ny, nz)
    std = {k: pkg.Storage(torch.from_numpy(v.astype(np.float32)).to(cuda), H) for k, v in {**inputs, **outs}.items()}
    pkg.call(name, std, sc32, domain=(nx, ny, nz))
    torch.cuda.synchronize()
    for a in spec.by_role("out3"):
        assert_bitwise_equal(dev[a.name].numpy(), std[a.name].numpy(), "%s.%s %s" % (name, a.name, size))


@pytest.mark.parametrize("name", NAMES)
def test_null_profile_is_refused(pkg, fields, cuda, name):
    import torch
    nx, ny, nz = 16, 12, 4
    spec, inputs, outs, sc, sc32 = _setup(pkg, fields, name, nx, ny, nz, 1, "physical")
    dev = {k: pkg.Storage(torch.from_numpy(v.astype(np.float32)).to(cuda), H) for k, v in {**inputs, **outs}.items()}
    lib = pkg.load_library()
    dom = pkg.Domain(nx, ny, nz)
    args = [ctypes.byref(dev[a.name].memref()) for a in spec.abi_args]
    base = torch.zeros(nz + 1, dtype=torch.float64, device=cuda)
    nb = len(pkg.kernels.PROFILED_FIELDS[name])
    for hole in range(nb):
        ptrs = [ctypes.c_void_p(0 if q == hole else base.data_ptr()) for q in range(nb)]
        scal = [ctypes.c_float(sc32[s.name]) for s in spec.scalars]
        rc = getattr(lib, "oeb_%s_f32_profiled" % name)(*args, *ptrs, *scal, ctypes.byref(dom), ctypes.c_void_p(0))
        assert rc == OEB_ERR_NULL, (name, hole, rc)
