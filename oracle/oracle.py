"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py use this
module, as the checker.  The product never imports it.

* :func:`run_oracle` calls ``liboeb_oracle.so``: the C restatement of the reference
  (oeb_oracle.c), built on every machine by ``oracle/build.py``.
* :func:`run_reference` calls ``oracle/_ref/liboeb_ref.so``: the reference's own headers,
  compiled from the reference source tree where that tree exists.

Both take numpy buffers keyed by the reference's argument names (whole allocations,
halo included, shape (nz+2h, ny+2h, nx+2h) or (n+2h,)), every argument of the reference
signature including scratch fields (allocated here when not given), the scalars and the
interior extents.  They write into the given buffers.
"""
from __future__ import annotations

import ctypes
from pathlib import Path
from typing import Dict, Optional

import numpy as np

from . import build as _build

ORACLE_SO = _build.ORACLE_SO
REF_SO = _build.REF_SO


class _M3(ctypes.Structure):
    _fields_ = [("allocated", ctypes.c_void_p), ("aligned", ctypes.c_void_p), ("offset", ctypes.c_int64),
                ("sizes", ctypes.c_int64 * 3), ("strides", ctypes.c_int64 * 3)]


class _M1(ctypes.Structure):
    _fields_ = [("allocated", ctypes.c_void_p), ("aligned", ctypes.c_void_p), ("offset", ctypes.c_int64),
                ("sizes", ctypes.c_int64 * 1), ("strides", ctypes.c_int64 * 1)]


def memref(arr: np.ndarray, halo: int):
    """Descriptor of a C-contiguous buffer in the reference layout (include/util.h:126-141)."""
    assert arr.flags.c_contiguous
    p = arr.ctypes.data
    if arr.ndim == 3:
        szk, szj, szi = arr.shape
        return _M3(p, p, halo * szj * szi + halo * szi + halo, (szk, szj, szi), (szj * szi, szi, 1))
    return _M1(p, p, halo, (arr.shape[0],), (1,))


_libs: Dict[str, ctypes.CDLL] = {}


def _lib(kind: str) -> ctypes.CDLL:
    if kind not in _libs:
        if kind == "oracle":
            path = _build.build_oracle()
        else:
            path = _build.build_ref() if not REF_SO.exists() else REF_SO
            if path is None or not Path(path).exists():
                raise FileNotFoundError("the reference harness needs the reference source tree (oracle/build.py)")
        _libs[kind] = ctypes.CDLL(str(path))
    return _libs[kind]


def reference_available() -> bool:
    if REF_SO.exists():
        return True
    try:
        return _build.build_ref() is not None
    except Exception:
        return False


def _args(spec, buffers: Dict[str, np.ndarray], halo: int, shape3, dtype):
    """ctypes arguments for every field of the reference signature, plus keep-alive list."""
    keep = []
    cargs = []
    for a in spec.args:
        arr = buffers.get(a.name)
        if arr is None:
            if a.role in ("in3", "in1", "out3"):
                raise ValueError("%s: missing buffer %r" % (spec.name, a.name))
            arr = np.zeros(shape3, dtype=dtype)  # scratch
            buffers[a.name] = arr
        if arr.dtype != dtype:
            raise TypeError("%s: buffer %r has dtype %s, expected %s" % (spec.name, a.name, arr.dtype, dtype))
        m = memref(arr, halo)
        keep.append(m)
        cargs.append(ctypes.byref(m))
    return cargs, keep


def _scalar_args(spec, scalars, f32: bool):
    out = []
    for s in spec.scalars:
        v = scalars[s.name]
        out.append(ctypes.c_double(v) if (not f32 or s.always_double) else ctypes.c_float(v))
    return out


def run_oracle(spec, buffers: Dict[str, np.ndarray], scalars: Dict[str, float], nx: int, ny: int, nz: int,
               halo: int) -> Dict[str, np.ndarray]:
    """Runs the C restatement of `spec` (oeb_oracle_<k>_{f64,f32}) in place on `buffers`."""
    dtype = next(iter(v.dtype for v in buffers.values()))
    f32 = dtype == np.float32
    shape3 = (nz + 2 * halo, ny + 2 * halo, nx + 2 * halo)
    cargs, keep = _args(spec, buffers, halo, shape3, dtype)
    fn = getattr(_lib("oracle"), "oeb_oracle_%s_%s" % (spec.name, "f32" if f32 else "f64"))
    fn.restype = None
    fn(*cargs, *_scalar_args(spec, scalars, f32), ctypes.c_int64(nx), ctypes.c_int64(ny), ctypes.c_int64(nz))
    del keep
    return buffers


VARIANT_IDS = {"default": 0, "fullfusion": 1, "partialfusion": 2, "openmp": 3}


def run_reference(spec, buffers: Dict[str, np.ndarray], scalars: Dict[str, float], n: int, nz: int, halo: int,
                  variant: str = "openmp") -> Dict[str, np.ndarray]:
    """Runs the reference's own kernel (square domain n x n x nz) in place on `buffers`.

    variant: default | fullfusion | partialfusion | openmp (include/util.h:10-13).  fvtp2d
    has no openmp variant; "openmp" runs its serial default there.
    """
    dtype = next(iter(v.dtype for v in buffers.values()))
    f32 = dtype == np.float32
    shape3 = (nz + 2 * halo, n + 2 * halo, n + 2 * halo)
    cargs, keep = _args(spec, buffers, halo, shape3, dtype)
    vid = VARIANT_IDS[variant]
    if spec.name == "fvtp2d" and variant != "fullfusion":
        vid = 0
    fn = getattr(_lib("ref"), "oeb_ref_%s_%s" % (spec.name, "f32" if f32 else "f64"))
    fn.restype = None
    fn(ctypes.c_int(vid), *cargs, *_scalar_args(spec, scalars, f32), ctypes.c_int64(n), ctypes.c_int64(nz))
    del keep
    return buffers
