"""The C ABI without a GPU: the library loads, exports exactly what include/oeb_gb300.h
declares, and rejects bad descriptors with the documented status before any CUDA call.

Descriptor validation runs on the host before a launch, so these calls return their error
status without touching a device (the pointers are never dereferenced).
"""
from __future__ import annotations

import ctypes
import subprocess

import numpy as np
import pytest

from conftest import ROOT

H = 3


def test_library_exports_every_declared_symbol(pkg):
    lib_path = pkg.LIB_PATH
    assert lib_path.exists()
    pkg.load_library()
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_path)], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    declared = set(pkg.declared_functions())
    assert declared, "no declarations parsed from include/oeb_gb300.h"
    missing = declared - exported
    assert not missing, "declared but not exported: %s" % sorted(missing)
    extra = {s for s in exported if s.startswith("oeb_")} - declared
    assert not extra, "exported but not declared: %s" % sorted(extra)


def test_every_kernel_has_device_and_host_entry_points(pkg):
    declared = set(pkg.declared_functions())
    for name in pkg.KERNELS:
        assert "oeb_%s_f64" % name in declared
        assert "oeb_%s_f64_host" % name in declared


def test_status_strings(pkg):
    lib = pkg.load_library()
    assert lib.oeb_status_string(0) == b"ok"
    for st in range(1, 13):
        assert lib.oeb_status_string(st) != b"unknown status"
    assert lib.oeb_status_string(99) == b"unknown status"
    assert lib.oeb_abi_version() >= 10000


def _fields(pkg, fields, name, nx=8, ny=8, nz=2, halo=H):
    inputs = fields.make_inputs(name, nx, ny, nz, seed=1, halo=halo)
    outs = fields.make_outputs(name, nx, ny, nz, halo=halo)
    return {k: pkg.Storage(v, halo) for k, v in {**inputs, **outs}.items()}


def _status(pkg, name, st, domain=(8, 8, 2), scalars=None, on_device=True):
    """Calls the device entry point with host memory; only validation can run here."""
    spec = pkg.KERNELS[name]
    cargs = [ctypes.byref(st[a.name].memref()) if st.get(a.name) is not None else None for a in spec.abi_args]
    vals = dict(pkg.DRIVER_SCALARS.get(name, {}))
    vals.update(scalars or {})
    for s in spec.scalars:
        cargs.append(ctypes.c_double(vals.get(s.name, 0.05)))
    dom = pkg.Domain(*domain)
    cargs += [ctypes.byref(dom), ctypes.c_void_p(0)]
    fn = getattr(pkg.load_library(), "oeb_%s_f64%s" % (name, "" if on_device else "_host"))
    fn.restype = ctypes.c_int
    return fn(*cargs)


@pytest.mark.parametrize("name", ("laplace", "hdiffsa", "hdiffsmag", "hadvuv", "hadvuv5th", "fastwavesuv",
                                  "uvbke", "nh_p_grad", "p_grad_c", "fvtp2d"))
def test_halo_too_small_is_rejected(pkg, fields, name):
    spec = pkg.KERNELS[name]
    need = spec.max_halo
    if need == 0:
        pytest.skip("no horizontal reach")
    st = _fields(pkg, fields, name, halo=need - 1 if need > 1 else 0)
    assert _status(pkg, name, st) == 4  # OEB_ERR_HALO


def test_null_descriptor_and_domain(pkg, fields):
    st = _fields(pkg, fields, "laplace")
    assert _status(pkg, "laplace", {"in": None, "out": st["out"]}) == 1  # OEB_ERR_NULL
    assert _status(pkg, "laplace", st, domain=(0, 8, 2)) == 2  # OEB_ERR_DOMAIN
    assert _status(pkg, "laplace", st, domain=(8, 8, -1)) == 2


def test_domain_larger_than_allocation_is_rejected(pkg, fields):
    st = _fields(pkg, fields, "laplace")
    assert _status(pkg, "laplace", st, domain=(11, 8, 2)) == 4  # nx + ihi beyond sizes[2] - hi
    assert _status(pkg, "laplace", st, domain=(8, 8, 6)) == 4  # nz + khi beyond sizes[0] - hk


def test_mismatched_strides_are_rejected(pkg, fields):
    st = _fields(pkg, fields, "laplace")
    other = pkg.Storage(np.zeros((2 + 2 * H, 8 + 2 * H, 24)), H, nx=8)  # padded pitch
    assert _status(pkg, "laplace", {"in": st["in"], "out": other}) == 3  # OEB_ERR_LAYOUT


def test_aliased_output_is_rejected(pkg, fields):
    st = _fields(pkg, fields, "laplace")
    assert _status(pkg, "laplace", {"in": st["in"], "out": st["in"]}) == 8  # OEB_ERR_ALIAS
    st2 = _fields(pkg, fields, "hdiffsmag")
    st2["vout"] = st2["uout"]
    assert _status(pkg, "hdiffsmag", st2) == 8


def test_non_unit_i_stride_is_rejected(pkg, fields):
    st = _fields(pkg, fields, "laplace")
    m = st["in"].memref()
    m.strides[2] = 2
    lib = pkg.load_library()
    dom = pkg.Domain(8, 8, 2)
    fn = lib.oeb_laplace_f64
    fn.restype = ctypes.c_int
    assert fn(ctypes.byref(m), ctypes.byref(st["out"].memref()), ctypes.byref(dom), None) == 3


def test_misaligned_pointer_is_rejected(pkg, fields):
    st = _fields(pkg, fields, "laplace")
    m = st["in"].memref()
    m.aligned = m.aligned + 4
    lib = pkg.load_library()
    dom = pkg.Domain(8, 8, 2)
    fn = lib.oeb_laplace_f64
    fn.restype = ctypes.c_int
    assert fn(ctypes.byref(m), ctypes.byref(st["out"].memref()), ctypes.byref(dom), None) == 5


def test_python_api_raises_on_errors(pkg, fields):
    st = _fields(pkg, fields, "laplace", halo=0)
    with pytest.raises(pkg.OebError) as e:
        pkg.call("laplace", st, {}, domain=(8, 8, 2))
    assert e.value.status == 4
    with pytest.raises(ValueError):
        pkg.call("laplace", {"in": st["in"]}, {}, domain=(8, 8, 2))


def test_storage_descriptor_matches_allocate_storage(pkg):
    """Storage.memref() builds allocateStorage's descriptor (include/util.h:126-141)."""
    n, nz, h = 10, 4, 3
    s = pkg.Storage.allocate3d(n, n, nz, h, device="host")
    m = s.memref()
    sz = [nz + 2 * h, n + 2 * h, n + 2 * h]
    assert list(m.sizes) == sz
    assert list(m.strides) == [sz[1] * sz[2], sz[2], 1]
    assert m.offset == h * m.strides[0] + h * m.strides[1] + h
    one = pkg.Storage.allocate1d(n, h, device="host")
    m1 = one.memref()
    assert (m1.offset, m1.sizes[0], m1.strides[0]) == (h, n + 2 * h, 1)


def test_variant_names_map_to_kernels(pkg):
    k = pkg.kernels
    for name, spec in pkg.KERNELS.items():
        for v in spec.variants:
            assert getattr(k, v) is getattr(k, name)
    assert len(pkg.VARIANTS) == 38  # 4 variants x 9 kernels + fvtp2d and fvtp2d_fullfusion
