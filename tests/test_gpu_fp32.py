"""FP32-storage stencils against the FP64 oracle, on the GPU, through the C ABI.

Two errors per output (normwise: max |e| / max |fp64| over the written box):

* ``arith``  -- the FP32 kernel against the FP64 oracle run on the SAME inputs rounded to
  FP32: the error of the FP32 arithmetic alone (exact sign tests, error-free products).
* ``total``  -- the FP32 kernel against the FP64 oracle on the original FP64 inputs: adds
  the quantisation of the inputs to FP32, which dominates wherever a stencil differences
  large, nearly equal values (pressure ~1000 with differences ~10 in nh_p_grad/p_grad_c).

The naive reference (the oracle's FP32 instantiation = the reference compiled with
ElementType = float, pinned by tests/golden/) is measured on the same inputs for comparison.
A limiter branch (hdiffsa, fvtp2d) can flip where the deciding difference is below FP32
resolution; such points are counted and bounded separately.
"""
from __future__ import annotations

import json
import os
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = 3
# Stated bounds (normwise).  arith: FP32 arithmetic alone.  total: including FP32 storage.
ARITH_TOL = 1e-6
TOTAL_TOL = {"laplace": 2e-5, "nh_p_grad": 6e-5, "p_grad_c": 6e-5}
TOTAL_TOL_DEFAULT = 1e-6
FLIP_KERNELS = {"hdiffsa"}          # limiter flips at input-resolution ties
FLIP_FRACTION = 1e-4                # at most 1 point in 10^4 above the bound
KERNELS = ("laplace", "hdiffsa", "hdiffsmag", "hadvuv", "hadvuv5th", "fastwavesuv", "uvbke", "nh_p_grad",
           "p_grad_c", "fvtp2d")
# the measured errors are also written, as JSON, to the file OEB_FP32_REPORT names (if set)
REPORT = Path(os.environ["OEB_FP32_REPORT"]) if os.environ.get("OEB_FP32_REPORT") else None
_results = {}


def _box(arr, reach, nx, ny, nz, h=H):
    ilo, ihi, jlo, jhi, klo, khi = reach
    return arr[h - klo:h + nz + khi, h - jlo:h + ny + jhi, h - ilo:h + nx + ihi]


def _run(pkg, fields, orc, cuda, name, nx, ny, nz, seed, workload):
    import torch
    spec = pkg.KERNELS[name]
    inputs = fields.make_inputs(name, nx, ny, nz, seed=seed, workload=workload)
    sc = fields.make_scalars(name, seed=seed)
    outs = fields.make_outputs(name, nx, ny, nz)
    sc32 = {s.name: (sc[s.name] if s.always_double else float(np.float32(sc[s.name]))) for s in spec.scalars}
    # FP64 oracle on the FP64 inputs, and on the inputs rounded to FP32
    ref = {k: v.copy() for k, v in {**inputs, **outs}.items()}
    orc.run_oracle(spec, ref, sc, nx, ny, nz, H)
    ref_q = {k: v.astype(np.float32).astype(np.float64) for k, v in {**inputs, **outs}.items()}
    orc.run_oracle(spec, ref_q, sc32, nx, ny, nz, H)
    naive = {k: v.astype(np.float32) for k, v in {**inputs, **outs}.items()}
    orc.run_oracle(spec, naive, sc32, nx, ny, nz, H)
    dev = {k: pkg.Storage(torch.from_numpy(v.astype(np.float32)).to(cuda), H) for k, v in {**inputs, **outs}.items()}
    pkg.call(name, dev, sc32, domain=(nx, ny, nz))
    torch.cuda.synchronize()
    res = {}
    for a in spec.by_role("out3"):
        want = _box(ref[a.name], a.reach, nx, ny, nz)
        want_q = _box(ref_q[a.name], a.reach, nx, ny, nz)
        got = _box(dev[a.name].numpy(), a.reach, nx, ny, nz).astype(np.float64)
        nai = _box(naive[a.name], a.reach, nx, ny, nz).astype(np.float64)
        scale = np.abs(want).max()
        e_tot = np.abs(got - want) / scale
        e_ar = np.abs(got - want_q) / scale
        e_nai = np.abs(nai - want_q) / scale
        res[a.name] = {"total_max": float(e_tot.max()), "total_rms": float(np.sqrt((e_tot ** 2).mean())),
                       "arith_max": float(e_ar.max()), "arith_rms": float(np.sqrt((e_ar ** 2).mean())),
                       "naive_arith_max": float(e_nai.max()),
                       "naive_arith_rms": float(np.sqrt((e_nai ** 2).mean())),
                       "points": int(e_tot.size),
                       "total_over_bound": int((e_tot > TOTAL_TOL.get(name, TOTAL_TOL_DEFAULT)).sum()),
                       "arith_over_bound": int((e_ar > ARITH_TOL).sum())}
        # cells outside the written box keep their value
        full = dev[a.name].numpy()
        mask = np.ones_like(full, dtype=bool)
        ilo, ihi, jlo, jhi, klo, khi = a.reach
        mask[H - klo:H + nz + khi, H - jlo:H + ny + jhi, H - ilo:H + nx + ihi] = False
        assert (full[mask] == np.float32(fields.SENTINEL)).all(), "%s.%s wrote outside its box" % (name, a.name)
    return res


@pytest.mark.parametrize("name", KERNELS)
@pytest.mark.parametrize("case", [("fronts", 256, 256, 80, 2), ("physical", 128, 128, 80, 1), ("fronts", 37, 45, 5, 9)])
def test_fp32_error_vs_fp64_oracle(pkg, fields, orc, cuda, name, case):
    workload, nx, ny, nz, seed = case
    res = _run(pkg, fields, orc, cuda, name, nx, ny, nz, seed, workload)
    _results["%s/%s_%dx%dx%d" % (name, workload, nx, ny, nz)] = res
    if REPORT is not None:
        REPORT.parent.mkdir(parents=True, exist_ok=True)
        REPORT.write_text(json.dumps(_results, indent=1, sort_keys=True))
    for out, r in res.items():
        what = "%s.%s %s" % (name, out, case)
        if name in FLIP_KERNELS:
            frac = max(r["total_over_bound"], r["arith_over_bound"]) / r["points"]
            assert frac <= FLIP_FRACTION, "%s: %.2g of points beyond the bound" % (what, frac)
            continue
        assert r["arith_max"] <= ARITH_TOL, "%s: arithmetic error %.3g" % (what, r["arith_max"])
        bound = TOTAL_TOL.get(name, TOTAL_TOL_DEFAULT)
        assert r["total_max"] <= bound, "%s: total error %.3g > %.1g" % (what, r["total_max"], bound)
        # the FP32 arithmetic is no worse than the naive float reference's (small margin)
        assert r["arith_max"] <= 2.0 * r["naive_arith_max"] + 1e-7, what


# FP32 stencils whose device-resident calls march k-levels with cp.async-staged tiles; with
# the fields in host memory (the host entry points in place) the plain tiled kernels run.
MARCHED = ("laplace", "hdiffsa", "nh_p_grad")


@pytest.mark.parametrize("name", MARCHED)
@pytest.mark.parametrize("size", [(256, 256, 80), (100, 70, 13), (37, 45, 5)], ids=["256x256x80", "100x70x13",
                                                                                 "37x45x5"])
@pytest.mark.parametrize("kb", [0, 1, 3])
def test_marched_forms_match_plain_kernels(pkg, fields, cuda, name, size, kb):
    """The staged march computes every output with the plain kernel's arithmetic on the same
    operands: the same bits, for the default k-blocking and forced ones (ragged chunks)."""
    import torch
    spec = pkg.KERNELS[name]
    nx, ny, nz = size
    lib = pkg.load_library()
    inputs = fields.make_inputs(name, nx, ny, nz, seed=11, workload="fronts")
    sc = fields.make_scalars(name, seed=11)
    sc32 = {s.name: (sc[s.name] if s.always_double else float(np.float32(sc[s.name]))) for s in spec.scalars}
    outs = fields.make_outputs(name, nx, ny, nz)
    arrays = {k: v.astype(np.float32) for k, v in {**inputs, **outs}.items()}
    assert lib.oeb_set_host_direct(1) == 0
    assert lib.oeb_set_kblock(kb) == 0
    try:
        host = {k: pkg.Storage(torch.from_numpy(v.copy()).pin_memory(), H) for k, v in arrays.items()}
        pkg.call(name, host, sc32, domain=(nx, ny, nz))
        dev = {k: pkg.Storage(torch.from_numpy(v.copy()).to(cuda), H) for k, v in arrays.items()}
        pkg.call(name, dev, sc32, domain=(nx, ny, nz))
        torch.cuda.synchronize()
    finally:
        lib.oeb_set_kblock(0)
    for a in spec.by_role("out3"):
        np.testing.assert_array_equal(dev[a.name].numpy().view(np.uint32), host[a.name].numpy().view(np.uint32),
                                      err_msg="%s.%s marched vs plain" % (name, a.name))


# The FP32 advection stencils, hdiffsmag and fastwavesuv run the reference's operation sequence
# in float, so they are bit-identical to the reference compiled for float (the oracle's float
# instantiation, pinned to that build by tests/golden/), in every tile shape (only the
# advection stencils have more than one).
@pytest.mark.parametrize("name", ("hadvuv", "hadvuv5th", "hdiffsmag", "fastwavesuv"))
@pytest.mark.parametrize("case", [("fronts", 256, 256, 80, 2), ("physical", 100, 70, 13, 5), ("fronts", 37, 45, 5, 9)])
@pytest.mark.parametrize("shape", [0, 1, 2])
def test_fp32_is_the_float_reference(pkg, fields, orc, cuda, name, case, shape):
    import torch
    if name not in ("hadvuv", "hadvuv5th") and shape:
        pytest.skip("%s has one tile shape" % name)
    workload, nx, ny, nz, seed = case
    spec = pkg.KERNELS[name]
    inputs = fields.make_inputs(name, nx, ny, nz, seed=seed, workload=workload)
    sc = fields.make_scalars(name, seed=seed)
    outs = fields.make_outputs(name, nx, ny, nz)
    sc32 = {s.name: float(np.float32(sc[s.name])) for s in spec.scalars}
    naive = {k: v.astype(np.float32) for k, v in {**inputs, **outs}.items()}
    orc.run_oracle(spec, naive, sc32, nx, ny, nz, H)
    lib = pkg.load_library()
    assert lib.oeb_set_tile_shape(shape) == 0
    try:
        dev = {k: pkg.Storage(torch.from_numpy(v.astype(np.float32)).to(cuda), H)
               for k, v in {**inputs, **outs}.items()}
        pkg.call(name, dev, sc32, domain=(nx, ny, nz))
        torch.cuda.synchronize()
    finally:
        lib.oeb_set_tile_shape(0)
    for a in spec.by_role("out3"):
        np.testing.assert_array_equal(dev[a.name].numpy().view(np.uint32), naive[a.name].view(np.uint32),
                                      err_msg="%s.%s %s shape %d vs the float reference" % (name, a.name, case, shape))
