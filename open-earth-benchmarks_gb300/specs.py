"""Argument tables of the ten stencils, in the order of the reference signatures.

Each kernel lists every argument of its ``kernels/<k>.h`` signature with a role:

* ``in3`` / ``in1`` -- a 3-D field / a 1-D per-latitude field the kernel reads;
* ``out3``          -- a 3-D field the kernel writes (its written box is ``box``);
* ``scratch3``      -- a 3-D work field of the reference signature; the GPU path neither
  reads nor writes it (it is not a parameter of the C ABI).

``reach`` is (ilo, ihi, jlo, jhi, klo, khi): cells touched beyond the interior on each side.
For inputs it is what the GPU kernel reads; for outputs the box it writes.  The same
numbers are checked by the C ABI (``csrc/k_*.cu``).

Scalars follow the fields in signature order.  ``dt5`` (uvbke) and ``p1``/``p2`` (fvtp2d)
are driver globals/macros in the reference (src/uvbke.cpp:11-12, src/fvtp2d.cpp:11-12); here
they are explicit scalars.  ``dt5`` is a double in every precision, as in the reference.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List, Tuple

Reach = Tuple[int, int, int, int, int, int]
INTERIOR: Reach = (0, 0, 0, 0, 0, 0)


@dataclass(frozen=True)
class Arg:
    name: str
    role: str  # in3 | in1 | out3 | scratch3
    reach: Reach = INTERIOR  # for in1 only (jlo, jhi) matter, stored in slots 2-3


@dataclass(frozen=True)
class Scalar:
    name: str
    always_double: bool = False


@dataclass(frozen=True)
class KernelSpec:
    name: str
    args: Tuple[Arg, ...]
    scalars: Tuple[Scalar, ...] = ()
    ref_header: str = ""
    oracle_variant: str = ""
    variants: Tuple[str, ...] = ()
    # interior points per call are nx*ny*nz; algorithmic bytes per point (FP64) =
    # (#in3 + #semantic out3) * 8, halo and 1-D fields excluded.
    semantic_outputs: Tuple[str, ...] = ()

    def by_role(self, role: str) -> List[Arg]:
        return [a for a in self.args if a.role == role]

    @property
    def abi_args(self) -> List[Arg]:
        """Arguments of the C ABI entry point (scratch fields dropped)."""
        return [a for a in self.args if a.role != "scratch3"]

    def bytes_per_point(self, elem_size: int = 8) -> int:
        return (len(self.by_role("in3")) + len(self.semantic_outputs)) * elem_size

    @property
    def max_halo(self) -> int:
        return max(max(a.reach[:4]) for a in self.args)


def _i(n, r=INTERIOR):
    return Arg(n, "in3", r)


def _l(n, jlo=0, jhi=0):
    return Arg(n, "in1", (0, 0, jlo, jhi, 0, 0))


def _o(n, r=INTERIOR):
    return Arg(n, "out3", r)


def _s(n):
    return Arg(n, "scratch3")


_VAR4 = ("{k}", "{k}_fullfusion", "{k}_partialfusion", "{k}_openmp")


def _variants(k):
    return tuple(v.format(k=k) for v in _VAR4)


_HADV_SCRATCH = tuple(_s(n) for n in ("uatupos", "vatupos", "uatvpos", "vatvpos", "uavg", "vavg", "ures", "vres"))

KERNELS: Dict[str, KernelSpec] = {}


def _add(spec: KernelSpec):
    KERNELS[spec.name] = spec


_add(KernelSpec(
    "laplace", (_i("in", (1, 1, 1, 1, 0, 0)), _o("out")),
    ref_header="kernels/laplace.h:4", oracle_variant="laplace_openmp (kernels/laplace.h:34-43)",
    variants=_variants("laplace"), semantic_outputs=("out",)))

_add(KernelSpec(
    "hdiffsa", (_o("out"), _i("in", (2, 2, 2, 2, 0, 0)), _i("mask"), _l("crlato", 1, 1), _l("crlatu", 1, 1),
                _s("lap"), _s("flx"), _s("fly")),
    ref_header="kernels/hdiffsa.h:4-5", oracle_variant="hdiffsa_openmp (kernels/hdiffsa.h:95-123)",
    variants=_variants("hdiffsa"), semantic_outputs=("out",)))

_add(KernelSpec(
    "hdiffsmag", (_o("uout"), _o("vout"), _i("uin", (1, 1, 1, 1, 0, 0)), _i("vin", (1, 1, 1, 1, 0, 0)), _i("mask"),
                  _l("crlavo"), _l("crlavu"), _l("crlato"), _l("crlatu"), _l("acrlat0", 1, 1), _s("T_sqr_s"),
                  _s("S_sqr_uv")),
    scalars=(Scalar("eddlat"), Scalar("eddlon"), Scalar("tau_smag"), Scalar("weight_smag")),
    ref_header="kernels/hdiffsmag.h:4-7", oracle_variant="hdiffsmag_openmp (kernels/hdiffsmag.h:205-263)",
    variants=_variants("hdiffsmag"), semantic_outputs=("uout", "vout")))

for _k, _h in (("hadvuv", 2), ("hadvuv5th", 3)):
    _add(KernelSpec(
        _k, (_o("uout"), _o("vout"), _i("uin", (_h,) * 4 + (0, 0)), _i("vin", (_h,) * 4 + (0, 0)), _l("acrlat0"),
             _l("acrlat1"), _l("tgrlatda0"), _l("tgrlatda1")) + _HADV_SCRATCH,
        scalars=(Scalar("eddlat"), Scalar("eddlon")),
        ref_header="kernels/hadvuv.h:29-32" if _k == "hadvuv" else "kernels/hadvuv5th.h:41-44",
        oracle_variant=("hadvuv_openmp (kernels/hadvuv.h:178-210)" if _k == "hadvuv"
                        else "hadvuv5th_openmp (kernels/hadvuv5th.h:177-201)"),
        variants=_variants(_k), semantic_outputs=("uout", "vout")))

_add(KernelSpec(
    "fastwavesuv", (_o("uout"), _o("vout"), _i("uin"), _i("vin"), _i("utens"), _i("vtens"),
                    _i("wgtfac", (0, 1, 0, 1, 0, 1)), _i("ppuv", (0, 1, 0, 1, 1, 1)), _i("hhl", (0, 1, 0, 1, 0, 1)),
                    _i("rho", (0, 1, 0, 1, 0, 0)), _l("fx"), _s("ppgk"), _s("ppgc"), _s("ppgu"), _s("ppgv")),
    scalars=(Scalar("edadlat"), Scalar("dt")),
    ref_header="kernels/fastwavesuv.h:4-7", oracle_variant="fastwavesuv_openmp (kernels/fastwavesuv.h:154-191)",
    variants=_variants("fastwavesuv"), semantic_outputs=("uout", "vout")))

_add(KernelSpec(
    "uvbke", (_o("ub"), _o("vb"), _i("uc", (0, 0, 1, 0, 0, 0)), _i("vc", (1, 0, 0, 0, 0, 0)), _i("cosa"),
              _i("rsina")),
    scalars=(Scalar("dt5", always_double=True),),
    ref_header="kernels/uvbke.h:4-5", oracle_variant="uvbke_openmp (kernels/uvbke.h:61-75)",
    variants=_variants("uvbke"), semantic_outputs=("ub", "vb")))

_add(KernelSpec(
    "nh_p_grad", (_o("uout"), _o("vout"), _i("uin"), _i("vin"), _i("rdx"), _i("rdy"), _i("gz", (0, 1, 0, 1, 0, 1)),
                  _i("pp", (0, 1, 0, 1, 0, 1)), _i("pk3", (0, 1, 0, 1, 0, 1)), _i("wk1", (0, 1, 0, 1, 0, 0)),
                  _s("wk"), _s("du"), _s("dv")),
    scalars=(Scalar("dt"),),
    ref_header="kernels/nh_p_grad.h:4-6", oracle_variant="nh_p_grad_openmp (kernels/nh_p_grad.h:116-146)",
    variants=_variants("nh_p_grad"), semantic_outputs=("uout", "vout")))

_add(KernelSpec(
    "p_grad_c", (_o("uout"), _o("vout"), _i("uin"), _i("vin"), _i("rdxc"), _i("rdyc"),
                 _i("delpc", (1, 0, 1, 0, 0, 0)), _i("gz", (1, 0, 1, 0, 0, 1)), _i("pkc", (1, 0, 1, 0, 0, 1)),
                 _s("wk")),
    scalars=(Scalar("dt2"),),
    ref_header="kernels/p_grad_c.h:4-6", oracle_variant="p_grad_c_openmp (kernels/p_grad_c.h:80-101)",
    variants=_variants("p_grad_c"), semantic_outputs=("uout", "vout")))

_FX = (0, 1, 3, 2, 0, 0)  # fx2 written / crx, xfx read: i in [0,N], j in [-3,N+1]
_FY = (3, 2, 0, 1, 0, 0)  # fy2 written / cry, yfx read: i in [-3,N+1], j in [0,N]
_add(KernelSpec(
    "fvtp2d", (_o("q_i", (3, 2, 0, 0, 0, 0)), _o("q_j", (0, 0, 3, 2, 0, 0)), _o("fx1"), _o("fx2", _FX), _o("fy1"),
               _o("fy2", _FY), _i("q", (3, 3, 3, 3, 0, 0)), _i("crx", _FX), _i("cry", _FY),
               _i("ra_x", (0, 0, 3, 2, 0, 0)), _i("ra_y", (3, 2, 0, 0, 0, 0)), _i("xfx", _FX), _i("yfx", _FY),
               _i("area", (3, 2, 3, 2, 0, 0)), _s("fxx"), _s("fyy"), _s("al"), _s("almq"), _s("br"), _s("b0"),
               _s("smt5")),
    scalars=(Scalar("p1"), Scalar("p2")),
    ref_header="kernels/fvtp2d.h:4-7", oracle_variant="fvtp2d (serial, kernels/fvtp2d.h:4-177)",
    variants=("fvtp2d", "fvtp2d_fullfusion"), semantic_outputs=("fx1", "fy1")))

KERNEL_NAMES = tuple(KERNELS)

# Scalar values of the reference drivers (src/<k>.cpp); dt5 and p1/p2 are the globals and
# macros of src/uvbke.cpp:11-12 and src/fvtp2d.cpp:11-12.
DRIVER_SCALARS = {
    "hdiffsmag": {"eddlat": 2.0 ** -11, "eddlon": 1.5 * 2.0 ** -11, "tau_smag": 0.025, "weight_smag": 0.01},
    "hadvuv": {"eddlat": 2.0 ** -11, "eddlon": 1.5 * 2.0 ** -11},
    "hadvuv5th": {"eddlat": 2.0 ** -11, "eddlon": 1.5 * 2.0 ** -11},
    "fastwavesuv": {"edadlat": 2.0 ** -11, "dt": 10.0},
    "uvbke": {"dt5": 0.5 * 225.0},
    "nh_p_grad": {"dt": 0.1},
    "p_grad_c": {"dt2": 0.1},
    "fvtp2d": {"p1": 0.583333, "p2": 0.083333},
}


# Tangent-linear / adjoint pairs: the active (differentiated) inputs of each stencil.  Every
# other input is a parameter held fixed.  The TL entry point oeb_<k>_tl_<p> takes
# (dy for every out3, the forward inputs, dx for each active input, scalars); the adjoint
# oeb_<k>_adj_<p> takes (xbar for each active input, the forward inputs, ybar for each
# semantic output, scalars).  xbar is written over the active input's reach box.
ACTIVE = {
    "hdiffsmag": ("uin", "vin"),
    "hadvuv": ("uin", "vin"),
    "hadvuv5th": ("uin", "vin"),
    "fastwavesuv": ("uin", "vin", "utens", "vtens", "ppuv"),
    "fvtp2d": ("q",),
    "laplace": ("in",),
    "hdiffsa": ("in",),
    "uvbke": ("uc", "vc"),
    "nh_p_grad": ("uin", "vin", "gz", "pp", "pk3", "wk1"),
    "p_grad_c": ("uin", "vin", "delpc", "gz", "pkc"),
}

# Fields an adjoint call reads or writes in full (frozen state and parameters it reads, the
# output seeds, the input gradients), for its algorithmic bytes: x elem size per point.
ADJ_FIELDS = {
    "hdiffsmag": ("uin", "vin", "mask", "uoutb", "voutb", "uinb", "vinb"),
    "hadvuv": ("uin", "vin", "uoutb", "voutb", "uinb", "vinb"),
    "hadvuv5th": ("uin", "vin", "uoutb", "voutb", "uinb", "vinb"),
    "fastwavesuv": ("wgtfac", "hhl", "rho", "uoutb", "voutb", "uinb", "vinb", "utensb", "vtensb", "ppuvb"),
    "fvtp2d": ("q", "crx", "cry", "ra_x", "ra_y", "xfx", "yfx", "area", "fx1b", "fy1b", "qb"),
    "laplace": ("outb", "inb"),
    "hdiffsa": ("in", "mask", "outb", "inb"),
    "uvbke": ("cosa", "rsina", "ubb", "vbb", "ucb", "vcb"),
    "nh_p_grad": ("rdx", "rdy", "gz", "pp", "pk3", "wk1", "uoutb", "voutb", "uinb", "vinb", "gzb", "ppb", "pk3b",
                  "wk1b"),
    "p_grad_c": ("rdxc", "rdyc", "delpc", "gz", "pkc", "uoutb", "voutb", "uinb", "vinb", "delpcb", "gzb", "pkcb"),
}
