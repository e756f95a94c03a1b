"""The reference's kernel functions, by name, over the GB300 library.

Every function of ``kernels/<k>.h`` is here with the same name and the same positional
arguments in the same order (include/oeb_gb300.h lists the signature each mirrors):
``laplace(in_, out)``, ``hdiffsa(out, in_, mask, crlato, crlatu, lap, flx, fly)``, ...,
plus the ``_fullfusion``, ``_partialfusion`` and ``_openmp`` variants, all of which run the
same GPU kernel (the oracle semantics of the reference's ``_openmp`` variant, serial
``fvtp2d`` for fvtp2d).  Fields are :class:`~.storage.Storage` objects.  The scratch
arguments of the reference signatures are accepted and ignored.

As in the reference, the interior extents are not arguments: they come from the module
globals ``domain_size`` and ``domain_height`` (src/<k>.cpp:4-5), unless a call passes
``domain=(nx, ny, nz)``.  Scalars that are driver globals in the reference (``dt5`` of
uvbke, ``p1``/``p2`` of fvtp2d) are keyword arguments with the drivers' values.

Fields on a CUDA device run asynchronously on ``stream`` (default: torch's current stream);
host fields go through the library's host entry points (synchronous, staged copies).
Errors raise :class:`~.abi.OebError`; nothing falls back to another implementation.
"""
from __future__ import annotations

import ctypes
from typing import Dict, Optional, Sequence

import numpy as np

from .abi import check, entry, load_library
from .specs import ACTIVE, DRIVER_SCALARS, KERNELS
from .storage import Domain, Storage

# Module globals of the reference drivers (src/<k>.cpp:4-6).
domain_size = 64
domain_height = 60
halo_width = 4


def _domain(domain) -> Domain:
    if domain is None:
        return Domain(domain_size, domain_size, domain_height)
    nx, ny, nz = domain
    return Domain(nx, ny, nz)


def _stream_handle(stream, on_device: bool) -> int:
    if stream is None:
        if not on_device:
            return 0
        import torch
        return torch.cuda.current_stream().cuda_stream
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


def set_adjoint_tiles(on: bool) -> None:
    """FP32 adjoints of hdiffsmag, hadvuv, hadvuv5th, fastwavesuv, p_grad_c and nh_p_grad as one tiled launch
    (True, the default) or in their multi-pass forms (oeb_set_adjoint_tiles); the same bits
    either way."""
    lib = load_library()
    check(lib.oeb_set_adjoint_tiles(ctypes.c_int(1 if on else 0)), "oeb_set_adjoint_tiles")


def entry_name(kernel: str, precision: str, on_device: bool) -> str:
    return "oeb_%s_%s%s" % (kernel, precision, "" if on_device else "_host")


def call(kernel: str, fields: Dict[str, Storage], scalars: Optional[Dict[str, float]] = None, domain=None,
         stream=None) -> None:
    """Runs `kernel` on named fields (the reference's argument names) and scalars."""
    spec = KERNELS[kernel]
    abi_args = spec.abi_args
    st = []
    for a in abi_args:
        f = fields.get(a.name)
        if f is None:
            raise ValueError("%s: missing field %r" % (kernel, a.name))
        if not isinstance(f, Storage):
            raise TypeError("%s: field %r must be a Storage" % (kernel, a.name))
        st.append(f)
    dtypes = {f.dtype for f in st}
    if len(dtypes) != 1:
        raise TypeError("%s: all fields must share one element type, got %s" % (kernel, sorted(map(str, dtypes))))
    precision = "f64" if st[0].dtype == np.float64 else "f32"
    places = {f.is_cuda for f in st}
    if len(places) != 1:
        raise ValueError("%s: fields must be all on the device or all in host memory" % kernel)
    on_device = places.pop()
    vals = dict(DRIVER_SCALARS.get(kernel, {}))
    vals.update(scalars or {})
    cargs = [ctypes.byref(f.memref()) for f in st]
    for s in spec.scalars:
        if s.name not in vals:
            raise ValueError("%s: missing scalar %r" % (kernel, s.name))
        ctype = ctypes.c_double if (precision == "f64" or s.always_double) else ctypes.c_float
        cargs.append(ctype(vals[s.name]))
    dom = _domain(domain)
    cargs += [ctypes.byref(dom), ctypes.c_void_p(_stream_handle(stream, on_device))]
    name = entry_name(kernel, precision, on_device)
    check(entry(name)(*cargs), name)


# The fields of the FP32 pressure-gradient stencils that the profiled entry points take as
# perturbations from an FP64 per-level base profile, in the entry points' argument order.
PROFILED_FIELDS = {"p_grad_c": ("gz", "pkc"), "nh_p_grad": ("gz", "pp", "pk3")}


def call_profiled(kernel: str, fields: Dict[str, Storage], bases, scalars: Optional[Dict[str, float]] = None,
                  domain=None, stream=None) -> None:
    """FP32 p_grad_c / nh_p_grad on profile-relative fields (oeb_<kernel>_f32_profiled).

    ``fields`` are FP32 device Storages as for :func:`call`, except that those named by
    ``PROFILED_FIELDS[kernel]`` hold perturbations: the field at interior level k is
    ``bases[name][k] + fields[name][k]``.  ``bases[name]`` is a float64 CUDA tensor of nz + 1
    values (interior levels 0 .. nz)."""
    if kernel not in PROFILED_FIELDS:
        raise ValueError("%s has no profiled form (only %s)" % (kernel, sorted(PROFILED_FIELDS)))
    spec = KERNELS[kernel]
    st = [fields[a.name] for a in spec.abi_args]
    if any(not isinstance(f, Storage) or not f.is_cuda or f.dtype != np.float32 for f in st):
        raise TypeError("%s: the profiled form takes FP32 device Storages" % kernel)
    dom = _domain(domain)
    ptrs = []
    for n in PROFILED_FIELDS[kernel]:
        b = bases[n]
        if not b.is_cuda or str(b.dtype) != "torch.float64" or b.numel() != dom.nz + 1 or not b.is_contiguous():
            raise ValueError("%s: base profile %r must be a contiguous float64 CUDA tensor of nz + 1 = %d values"
                             % (kernel, n, dom.nz + 1))
        ptrs.append(ctypes.c_void_p(b.data_ptr()))
    vals = dict(DRIVER_SCALARS.get(kernel, {}))
    vals.update(scalars or {})
    cargs = [ctypes.byref(f.memref()) for f in st] + ptrs + _scalar_args(spec, vals, "f32")
    cargs += [ctypes.byref(dom), ctypes.c_void_p(_stream_handle(stream, True))]
    name = "oeb_%s_f32_profiled" % kernel
    check(entry(name)(*cargs), name)


def _scalar_args(spec, vals, precision):
    out = []
    for s in spec.scalars:
        if s.name not in vals:
            raise ValueError("%s: missing scalar %r" % (spec.name, s.name))
        ctype = ctypes.c_double if (precision == "f64" or s.always_double) else ctypes.c_float
        out.append(ctype(vals[s.name]))
    return out


def _device_fields(kernel, groups):
    flat = [f for g in groups for f in g]
    if any(not isinstance(f, Storage) for f in flat):
        raise TypeError("%s: every field must be a Storage" % kernel)
    if not all(f.is_cuda for f in flat):
        raise ValueError("%s: the tangent-linear and adjoint entry points take device fields" % kernel)
    dtypes = {f.dtype for f in flat}
    if len(dtypes) != 1:
        raise TypeError("%s: mixed element types" % kernel)
    return "f64" if flat[0].dtype == np.float64 else "f32"


def tangent_linear(kernel: str, state: Dict[str, Storage], dx: Dict[str, Storage], dy: Dict[str, Storage],
                   scalars: Optional[Dict[str, float]] = None, domain=None, stream=None) -> None:
    """dy = J(state) dx: the stencil's Jacobian at `state` (branches frozen) applied to dx.

    dx holds a perturbation of each active input (ACTIVE[kernel]); dy receives the
    perturbation of every output, over the output's written box."""
    spec = KERNELS[kernel]
    outs = [dy[a.name] for a in spec.by_role("out3")]
    ins = [state[a.name] for a in spec.args if a.role in ("in3", "in1")]
    dxs = [dx[n] for n in ACTIVE[kernel]]
    precision = _device_fields(kernel, (outs, ins, dxs))
    vals = dict(DRIVER_SCALARS.get(kernel, {}))
    vals.update(scalars or {})
    cargs = [ctypes.byref(f.memref()) for f in outs + ins + dxs] + _scalar_args(spec, vals, precision)
    dom = _domain(domain)
    cargs += [ctypes.byref(dom), ctypes.c_void_p(_stream_handle(stream, True))]
    name = "oeb_%s_tl_%s" % (kernel, precision)
    check(entry(name)(*cargs), name)


def adjoint(kernel: str, state: Dict[str, Storage], ybar: Dict[str, Storage], xbar: Dict[str, Storage],
            scalars: Optional[Dict[str, float]] = None, domain=None, stream=None) -> None:
    """xbar = J(state)^T ybar for the active inputs; ybar seeds the semantic outputs."""
    spec = KERNELS[kernel]
    xbs = [xbar[n] for n in ACTIVE[kernel]]
    ins = [state[a.name] for a in spec.args if a.role in ("in3", "in1")]
    ybs = [ybar[n] for n in spec.semantic_outputs]
    precision = _device_fields(kernel, (xbs, ins, ybs))
    vals = dict(DRIVER_SCALARS.get(kernel, {}))
    vals.update(scalars or {})
    cargs = [ctypes.byref(f.memref()) for f in xbs + ins + ybs] + _scalar_args(spec, vals, precision)
    dom = _domain(domain)
    cargs += [ctypes.byref(dom), ctypes.c_void_p(_stream_handle(stream, True))]
    name = "oeb_%s_adj_%s" % (kernel, precision)
    check(entry(name)(*cargs), name)


def _make(kernel: str):
    spec = KERNELS[kernel]
    names = [a.name for a in spec.args]
    scalar_names = [s.name for s in spec.scalars]

    def fn(*args, domain=None, stream=None, **kw):
        n_fields = len(names)
        if len(args) < n_fields:
            # trailing scratch arguments may be omitted
            args = list(args) + [None] * (n_fields - len(args))
        fields = dict(zip(names, args[:n_fields]))
        extra = list(args[n_fields:])
        scal = {}
        for sname in scalar_names:
            if extra:
                scal[sname] = extra.pop(0)
        if extra:
            raise TypeError("%s: too many positional arguments" % kernel)
        scal.update({k: v for k, v in kw.items() if k in {s.name for s in spec.scalars}})
        unknown = set(kw) - {s.name for s in spec.scalars}
        if unknown:
            raise TypeError("%s: unexpected keyword arguments %s" % (kernel, sorted(unknown)))
        call(kernel, {k: v for k, v in fields.items() if v is not None}, scal, domain=domain, stream=stream)

    fn.__name__ = kernel
    fn.__doc__ = "%s(%s) -- %s; oracle semantics of %s." % (kernel, ", ".join(names + scalar_names),
                                                            spec.ref_header, spec.oracle_variant)
    return fn


laplace = _make("laplace")
hdiffsa = _make("hdiffsa")
hdiffsmag = _make("hdiffsmag")
hadvuv = _make("hadvuv")
hadvuv5th = _make("hadvuv5th")
fastwavesuv = _make("fastwavesuv")
uvbke = _make("uvbke")
nh_p_grad = _make("nh_p_grad")
p_grad_c = _make("p_grad_c")
fvtp2d = _make("fvtp2d")

# The reference's variants (util.h:10-13) name the same computation; each runs the one GPU
# kernel.  fvtp2d_fullfusion reads a stale scratch value in the reference
# (kernels/fvtp2d.h:195-196); here it runs the faithful serial fvtp2d.
VARIANTS: Dict[str, str] = {}
for _k, _spec in KERNELS.items():
    for _v in _spec.variants:
        VARIANTS[_v] = _k
        if _v != _k:
            globals()[_v] = globals()[_k]


def variant_kernel(name: str) -> str:
    return VARIANTS[name]


__all__ = ["call", "tangent_linear", "adjoint", "domain_size", "domain_height", "halo_width", "VARIANTS", "variant_kernel",
           *KERNELS.keys(), *[v for v in VARIANTS if v not in KERNELS]]
