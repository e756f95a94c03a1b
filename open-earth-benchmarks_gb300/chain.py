"""The chained dycore step and CUDA graphs (the ``oeb_chain_*`` / ``oeb_graph_*`` C ABI).

One step maps (u, v) to (uout, vout, fx1, fy1) through fastwavesuv, hadvuv5th, an explicit
update u2 = u1 + dt_adv * (advective tendency), hdiffsmag and fvtp2d (the PPM fluxes of the
new u); include/oeb_gb300.h states the stages and boxes.  The tangent-linear and adjoint
steps recompute the intermediate states inside the call.

    plan = ChainPlan(like=fields["u"], domain=(nx, ny, nz), modes=FORWARD | ADJOINT)
    plan.forward(fields, scalars, outs)            # outs: uout, vout, fx1, fy1
    plan.adjoint(fields, scalars, seeds, grads)    # seeds: uout, vout, fx1, fy1 -> grads: u, v
    with Graph(stream) as g:                       # record library calls ...
        plan.forward(fields, scalars, outs, stream=stream)
    g.launch(stream)                               # ... and replay them

Every 3-D field of a step shares the layout of ``like`` (sizes, strides and offset) with an
i/j halo of at least 8 and a k halo of at least 1.
"""
from __future__ import annotations

import ctypes
import json
from typing import Dict, List, Optional, Tuple

import numpy as np

from .abi import OebError, check, entry, load_library
from .storage import Domain, Memref1d, Memref3d, Storage

FORWARD, TL, ADJOINT = 1, 2, 4
FUSE_HADV_UPDATE = 1  # hadvuv5th and the explicit update as one kernel (oeb_set_fusion)
HALO = 8  # i/j halo the step's inputs need

FIELDS3 = ("u", "v", "utens", "vtens", "wgtfac", "ppuv", "hhl", "rho")
ORDER = ("u", "v", "utens", "vtens", "wgtfac", "ppuv", "hhl", "rho", "fx", "acrlat0", "acrlat1", "tgrlatda0",
         "tgrlatda1", "mask", "crlavo", "crlavu", "crlato", "crlatu", "smag_acrlat0", "crx", "cry", "ra_x", "ra_y",
         "xfx", "yfx", "area")
RANK1 = {"fx", "acrlat0", "acrlat1", "tgrlatda0", "tgrlatda1", "crlavo", "crlavu", "crlato", "crlatu",
         "smag_acrlat0"}
SCALARS = ("edadlat", "dt", "eddlat", "eddlon", "dt_adv", "tau_smag", "weight_smag", "ppm_p1", "ppm_p2")
OUTPUTS = ("uout", "vout", "fx1", "fy1")


def set_fusion(mask: int) -> None:
    """The fusion grouping of every later single chained step (oeb_set_fusion):
    FUSE_HADV_UPDATE (the default) runs hadvuv5th and the explicit update as one kernel, 0 runs
    each stage as its own kernels.  Results do not depend on it."""
    check(entry("oeb_set_fusion")(ctypes.c_int(mask)), "oeb_set_fusion")


class ChainFields(ctypes.Structure):
    """oeb_chain_fields_{f64,f32}: one descriptor pointer per input, in ORDER."""
    _fields_ = [(n, ctypes.POINTER(Memref1d if n in RANK1 else Memref3d)) for n in ORDER]


class ChainScalars(ctypes.Structure):
    """oeb_chain_scalars."""
    _fields_ = [(n, ctypes.c_double) for n in SCALARS]


def _precision(fields) -> str:
    kinds = {f.dtype for f in fields}
    if len(kinds) != 1:
        raise TypeError("the fields of a step share one element type")
    return "f64" if next(iter(kinds)) == np.float64 else "f32"


def _stream(stream) -> int:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


class ChainPlan:
    """Workspace of the chained step for one layout and domain (oeb_chain_plan_create_*)."""

    def __init__(self, like: Storage, domain, modes: int = FORWARD):
        self.precision = "f64" if like.dtype == np.float64 else "f32"
        self.domain = Domain(*domain)
        self._plan = ctypes.c_void_p()
        fn = entry("oeb_chain_plan_create_%s" % self.precision)
        check(fn(ctypes.byref(like.memref()), ctypes.byref(self.domain), ctypes.c_int(modes),
                 ctypes.byref(self._plan)), "oeb_chain_plan_create")
        self.modes = modes
        self._keep = []

    @property
    def nbytes(self) -> int:
        lib = load_library()
        lib.oeb_chain_plan_bytes.restype = ctypes.c_size_t
        lib.oeb_chain_plan_bytes.argtypes = [ctypes.c_void_p]
        return int(lib.oeb_chain_plan_bytes(self._plan))

    def close(self):
        if self._plan:
            lib = load_library()
            lib.oeb_chain_plan_destroy.argtypes = [ctypes.c_void_p]
            check(lib.oeb_chain_plan_destroy(self._plan), "oeb_chain_plan_destroy")
            self._plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _fields(self, fields: Dict[str, Storage]):
        missing = [n for n in ORDER if n not in fields]
        if missing:
            raise ValueError("chain step: missing fields %s" % missing)
        refs = {n: fields[n].memref() for n in ORDER}
        cf = ChainFields(**{n: ctypes.pointer(refs[n]) for n in ORDER})
        self._keep = [refs, cf]  # alive until the next call; a captured graph copies them at capture
        return cf

    @staticmethod
    def _scalars(scalars: Dict[str, float]) -> ChainScalars:
        missing = [n for n in SCALARS if n not in scalars]
        if missing:
            raise ValueError("chain step: missing scalars %s" % missing)
        return ChainScalars(**{n: float(scalars[n]) for n in SCALARS})

    def _call(self, what, fields, scalars, extra, stream):
        prec = _precision([fields[n] for n in ORDER] + list(extra))
        if prec != self.precision:
            raise TypeError("the plan is %s, the fields are %s" % (self.precision, prec))
        cf = self._fields(fields)
        cs = self._scalars(scalars)
        refs = [f.memref() for f in extra]
        args = [self._plan, ctypes.byref(cf), ctypes.byref(cs)] + [ctypes.byref(r) for r in refs]
        name = "oeb_chain_%s_%s" % (what, self.precision)
        check(entry(name)(*args, ctypes.c_void_p(_stream(stream))), name)

    def forward(self, fields, scalars, outs: Dict[str, Storage], stream=None):
        self._call("forward", fields, scalars, [outs[n] for n in OUTPUTS], stream)

    def tangent_linear(self, fields, scalars, dx: Dict[str, Storage], dy: Dict[str, Storage], stream=None):
        self._call("tl", fields, scalars, [dx["u"], dx["v"]] + [dy[n] for n in OUTPUTS], stream)

    def adjoint(self, fields, scalars, seeds: Dict[str, Storage], grads: Dict[str, Storage], stream=None):
        self._call("adj", fields, scalars, [seeds[n] for n in OUTPUTS] + [grads["u"], grads["v"]], stream)


class Graph:
    """A CUDA graph of library calls made on `stream` inside the ``with`` block."""

    def __init__(self, stream):
        self.stream = stream
        self._g = ctypes.c_void_p()

    def __enter__(self):
        check(entry("oeb_graph_begin")(ctypes.c_void_p(_stream(self.stream))), "oeb_graph_begin")
        return self

    def __exit__(self, exc_type, exc, tb):
        st = entry("oeb_graph_end")(ctypes.c_void_p(_stream(self.stream)), ctypes.byref(self._g))
        if exc_type is None:
            check(st, "oeb_graph_end")
        return False

    @property
    def kernels(self) -> int:
        lib = load_library()
        lib.oeb_graph_kernel_count.restype = ctypes.c_uint64
        lib.oeb_graph_kernel_count.argtypes = [ctypes.c_void_p]
        return int(lib.oeb_graph_kernel_count(self._g))

    def launch(self, stream=None):
        s = self.stream if stream is None else stream
        check(entry("oeb_graph_launch")(self._g, ctypes.c_void_p(_stream(s))), "oeb_graph_launch")

    def close(self):
        if self._g:
            entry("oeb_graph_destroy")(self._g)
            self._g = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchMember(ctypes.Structure):
    """oeb_batch_member."""
    _fields_ = [("elem_size", ctypes.c_int), ("dom", Domain), ("fields", ctypes.c_void_p), ("scalars", ChainScalars),
                ("uout", ctypes.c_void_p), ("vout", ctypes.c_void_p), ("fx1", ctypes.c_void_p),
                ("fy1", ctypes.c_void_p), ("uoutb", ctypes.c_void_p), ("voutb", ctypes.c_void_p),
                ("fx1b", ctypes.c_void_p), ("fy1b", ctypes.c_void_p), ("ub", ctypes.c_void_p), ("vb", ctypes.c_void_p)]


class BatchPlan:
    """The chained step of many ensemble members as batched persistent launches
    (oeb_batch_plan_create / oeb_batch_run / oeb_batch_autotune).

    members: a list of dicts with keys ``fields`` (the step's inputs, as for ChainPlan),
    ``scalars``, ``domain`` (nx, ny, nz), ``outs`` (uout, vout, fx1, fy1) and, for the
    adjoint, ``seeds`` (uout, vout, fx1, fy1) and ``grads`` (u, v).  FP64 and FP32 members
    may be mixed.  The descriptors are copied at creation: every run reads and writes the
    same buffers."""

    def __init__(self, members, modes: int = FORWARD | ADJOINT):
        keep = []
        arr = (BatchMember * len(members))()
        for i, m in enumerate(members):
            f = m["fields"]
            refs = {n: f[n].memref() for n in ORDER}
            cf = ChainFields(**{n: ctypes.pointer(refs[n]) for n in ORDER})
            keep += [refs, cf]
            b = arr[i]
            b.elem_size = f["u"].dtype.itemsize
            b.dom = Domain(*m["domain"])
            b.fields = ctypes.cast(ctypes.pointer(cf), ctypes.c_void_p)
            b.scalars = ChainPlan._scalars(m["scalars"])
            io = {}
            for n in OUTPUTS:
                io[n] = m["outs"][n] if "outs" in m else None
                io[n + "b"] = m["seeds"][n] if "seeds" in m else None
            io["ub"] = m["grads"]["u"] if "grads" in m else None
            io["vb"] = m["grads"]["v"] if "grads" in m else None
            for n, st in io.items():
                if st is not None:
                    r = st.memref()
                    keep.append(r)
                    setattr(b, n, ctypes.cast(ctypes.pointer(r), ctypes.c_void_p))
        self._plan = ctypes.c_void_p()
        check(entry("oeb_batch_plan_create")(arr, ctypes.c_int(len(members)), ctypes.c_int(modes),
                                             ctypes.byref(self._plan)), "oeb_batch_plan_create")
        del keep

    def run(self, stream=None):
        check(entry("oeb_batch_run")(self._plan, ctypes.c_void_p(_stream(stream))), "oeb_batch_run")

    def autotune(self, stream=None):
        check(entry("oeb_batch_autotune")(self._plan, ctypes.c_void_p(_stream(stream))), "oeb_batch_autotune")

    TUNING_FORMAT = "oeb-batch-tuning/3"

    @property
    def signature(self) -> int:
        """64-bit hash of the modes, the members' element sizes and domains, and the launch
        count (oeb_batch_signature): a tuning record fits every plan with the same one."""
        out = ctypes.c_uint64()
        check(entry("oeb_batch_signature")(self._plan, ctypes.byref(out)), "oeb_batch_signature")
        return int(out.value)

    def tuning(self) -> List[Tuple[int, int, int]]:
        """The plan's launch choices, (kb, tile shape, form) per batched launch in run order
        (oeb_batch_tuning_get); shape 0 is 32 x 32 cells a CTA, 1 32 x 8, 2 64 x 16 (for the
        kernels that take one); form 0 is one persistent wave, 1 one CTA per tile, 2 one
        ordinary launch per member."""
        n = ctypes.c_int()
        check(entry("oeb_batch_tuning_get")(self._plan, None, ctypes.c_int(0), ctypes.byref(n)),
              "oeb_batch_tuning_get")
        rec = (ctypes.c_int * (3 * max(n.value, 1)))()
        check(entry("oeb_batch_tuning_get")(self._plan, rec, n, ctypes.byref(n)), "oeb_batch_tuning_get")
        return [(rec[3 * i], rec[3 * i + 1], rec[3 * i + 2]) for i in range(n.value)]

    def apply_tuning(self, choices) -> None:
        """Makes the plan launch as `choices` says (oeb_batch_tuning_apply): as tuning()
        returns them, here or in another process, for a plan with the same signature."""
        choices = [tuple(c) for c in choices]
        if any(len(c) != 3 for c in choices):
            raise OebError("a tuning choice is (kb, shape, form)", 12)
        flat = [int(v) for c in choices for v in c]
        rec = (ctypes.c_int * max(len(flat), 1))(*flat)
        check(entry("oeb_batch_tuning_apply")(self._plan, rec, ctypes.c_int(len(flat) // 3)),
              "oeb_batch_tuning_apply")

    @property
    def fusion(self) -> int:
        """The fusion grouping the plan's launches were recorded with (FUSE_* bits)."""
        m = ctypes.c_int()
        check(entry("oeb_batch_get_fusion")(self._plan, ctypes.byref(m)), "oeb_batch_get_fusion")
        return int(m.value)

    def set_fusion(self, mask: int) -> None:
        """Records the step again with fusion grouping `mask` and the default choices."""
        check(entry("oeb_batch_set_fusion")(self._plan, ctypes.c_int(mask)), "oeb_batch_set_fusion")

    def save_tuning(self, path) -> None:
        """Writes the plan's fusion grouping and choices as a JSON tuning record, keyed by its
        signature."""
        with open(path, "w") as f:
            json.dump({"format": self.TUNING_FORMAT, "signature": "%016x" % self.signature,
                       "fusion": self.fusion, "choices": [list(c) for c in self.tuning()]}, f)

    def load_tuning(self, path) -> None:
        """Applies a record written by save_tuning.  Raises OebError, leaving the plan as it
        was, if the record is of another format or was saved for a plan with another
        signature (other members, domains, precisions or modes)."""
        with open(path) as f:
            rec = json.load(f)
        if rec.get("format") != self.TUNING_FORMAT:
            raise OebError("%s: not a batch tuning record (format %r)" % (path, rec.get("format")))
        if rec.get("signature") != "%016x" % self.signature:
            raise OebError("%s: saved for another ensemble (signature %s, this plan %016x)"
                           % (path, rec.get("signature"), self.signature))
        if self.fusion != rec.get("fusion", 0):
            self.set_fusion(int(rec.get("fusion", 0)))
        self.apply_tuning(rec["choices"])

    # launch forms (oeb_batch_set_form)
    PER_LAUNCH, ONE_LAUNCH = 0, 1

    def set_form(self, form: int, kb: int = 0, ctas_per_sm: int = 2) -> None:
        """Runs the plan as one launch per recorded position and precision (PER_LAUNCH, the
        default) or as ONE persistent launch of the step kernel (ONE_LAUNCH, its tasks
        recorded with k-blocking kb: 0 = each kernel's default, 1, 2, 4, 8; the kernel built
        for ctas_per_sm = 2, 3 or 4 CTAs an SM)."""
        check(entry("oeb_batch_set_form")(self._plan, ctypes.c_int(form), ctypes.c_int(kb), ctypes.c_int(ctas_per_sm)),
              "oeb_batch_set_form")

    @property
    def form(self) -> Tuple[int, int, int]:
        """(form, kb, ctas_per_sm); kb and ctas_per_sm are -1 for the per-launch form."""
        f, kb, n = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(entry("oeb_batch_get_form")(self._plan, ctypes.byref(f), ctypes.byref(kb), ctypes.byref(n)),
              "oeb_batch_get_form")
        return int(f.value), int(kb.value), int(n.value)

    def step_waits(self) -> Tuple[int, int]:
        """(microseconds, count) of the last one-launch run's waits that had to poll, summed
        over its CTAs.  Waits for the device to go idle."""
        us, n = ctypes.c_uint64(), ctypes.c_uint64()
        check(entry("oeb_batch_step_waits")(self._plan, ctypes.byref(us), ctypes.byref(n)), "oeb_batch_step_waits")
        return int(us.value), int(n.value)

    def autotune_form(self, stream=None) -> float:
        """Times whole runs of the per-launch form as it stands and of the one-launch form
        with each kb, keeps the fastest, and returns its milliseconds per run."""
        ms = ctypes.c_float()
        check(entry("oeb_batch_autotune_form")(self._plan, ctypes.c_void_p(_stream(stream)), ctypes.byref(ms)),
              "oeb_batch_autotune_form")
        return float(ms.value)

    def step_status(self) -> Tuple[int, int]:
        """(status, task) of the last one-launch run: (0, -1), or (OEB_ERR_TIMEOUT, the task
        whose wait gave up).  Waits for the device to go idle."""
        st, task = ctypes.c_int(), ctypes.c_int()
        check(entry("oeb_batch_step_status")(self._plan, ctypes.byref(st), ctypes.byref(task)),
              "oeb_batch_step_status")
        return int(st.value), int(task.value)

    def set_wait_limit(self, ns: int) -> None:
        """The longest one wait of the step kernel may last, in nanoseconds."""
        check(entry("oeb_batch_set_wait_limit")(self._plan, ctypes.c_uint64(ns)), "oeb_batch_set_wait_limit")

    def withhold(self, on: bool) -> None:
        """Test hook: the first task of the one-launch form waits for a count that nothing
        writes (on), so the next run ends with OEB_ERR_TIMEOUT; off restores it."""
        check(entry("oeb_batch_withhold")(self._plan, ctypes.c_int(1 if on else 0)), "oeb_batch_withhold")

    @property
    def launches(self) -> int:
        return int(entry("oeb_batch_launches")(self._plan))

    @property
    def points(self) -> int:
        lib = load_library()
        lib.oeb_batch_points.restype = ctypes.c_int64
        lib.oeb_batch_points.argtypes = [ctypes.c_void_p]
        return int(lib.oeb_batch_points(self._plan))

    @property
    def nbytes(self) -> int:
        lib = load_library()
        lib.oeb_batch_plan_bytes.restype = ctypes.c_size_t
        lib.oeb_batch_plan_bytes.argtypes = [ctypes.c_void_p]
        return int(lib.oeb_batch_plan_bytes(self._plan))

    def close(self):
        if self._plan:
            lib = load_library()
            lib.oeb_batch_plan_destroy.argtypes = [ctypes.c_void_p]
            check(lib.oeb_batch_plan_destroy(self._plan), "oeb_batch_plan_destroy")
            self._plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
