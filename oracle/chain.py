"""The chained dycore step composed from the oracle's stencils (TEST INFRASTRUCTURE).

Only tests/ and bench.py's CPU leg use this, as the checker.  The step is the one of
open-earth-benchmarks_gb300/chain.py: fastwavesuv over the interior widened by 7 cells in
i and j, hadvuv5th widened by 4, u2 = u1 + dt_adv * tendency on the same box, hdiffsmag
widened by 3, fvtp2d of the new u on the interior.  Each widened stage is an ordinary
oracle call on a view of the same buffers: with an i/j halo of H, the view that drops e
k-planes at each end has a halo of H - e on every axis, and its interior is the original
interior widened by e in i and j.
"""
from __future__ import annotations

from typing import Dict

import numpy as np

from . import oracle

E1, E2, E3 = 7, 4, 3
SENTINEL = -7.0e5


def _kview(arr: np.ndarray, e: int) -> np.ndarray:
    return arr[e:arr.shape[0] - e] if arr.ndim == 3 else arr


def _stage(kernel: str, buffers: Dict[str, np.ndarray], scalars, nx, ny, nz, halo, e):
    from oeb_gb300.specs import KERNELS  # the argument table the oracle calls are built from
    views = {k: _kview(v, e) for k, v in buffers.items()}
    oracle.run_oracle(KERNELS[kernel], views, scalars, nx + 2 * e, ny + 2 * e, nz, halo - e)


def run_chain(x: Dict[str, np.ndarray], s: Dict[str, float], nx: int, ny: int, nz: int, halo: int) -> Dict[str, np.ndarray]:
    """Outputs uout, vout (written over the interior widened by 3), fx1, fy1 (interior) and
    the intermediates u1, v1, tu, tv, u2, v2, of the step at inputs x (whole buffers)."""
    if halo < E1 + 1:
        raise ValueError("the chained step needs an i/j halo of at least 8")
    dtype = x["u"].dtype
    shape = x["u"].shape
    new = lambda: np.full(shape, SENTINEL, dtype=dtype)  # noqa: E731
    o = {n: new() for n in ("u1", "v1", "tu", "tv", "u2", "v2", "uout", "vout", "q_i", "q_j", "fx1", "fx2", "fy1",
                           "fy2")}
    _stage("fastwavesuv", {"uout": o["u1"], "vout": o["v1"], "uin": x["u"], "vin": x["v"], "utens": x["utens"],
                           "vtens": x["vtens"], "wgtfac": x["wgtfac"], "ppuv": x["ppuv"], "hhl": x["hhl"],
                           "rho": x["rho"], "fx": x["fx"]},
           {"edadlat": s["edadlat"], "dt": s["dt"]}, nx, ny, nz, halo, E1)
    _stage("hadvuv5th", {"uout": o["tu"], "vout": o["tv"], "uin": o["u1"], "vin": o["v1"], "acrlat0": x["acrlat0"],
                         "acrlat1": x["acrlat1"], "tgrlatda0": x["tgrlatda0"], "tgrlatda1": x["tgrlatda1"]},
           {"eddlat": s["eddlat"], "eddlon": s["eddlon"]}, nx, ny, nz, halo, E2)
    box = (slice(halo, halo + nz), slice(halo - E2, halo + ny + E2), slice(halo - E2, halo + nx + E2))
    dt_adv = dtype.type(s["dt_adv"])
    o["u2"][box] = o["u1"][box] + dt_adv * o["tu"][box]
    o["v2"][box] = o["v1"][box] + dt_adv * o["tv"][box]
    _stage("hdiffsmag", {"uout": o["uout"], "vout": o["vout"], "uin": o["u2"], "vin": o["v2"], "mask": x["mask"],
                         "crlavo": x["crlavo"], "crlavu": x["crlavu"], "crlato": x["crlato"], "crlatu": x["crlatu"],
                         "acrlat0": x["smag_acrlat0"]},
           {"eddlat": s["eddlat"], "eddlon": s["eddlon"], "tau_smag": s["tau_smag"],
            "weight_smag": s["weight_smag"]}, nx, ny, nz, halo, E3)
    _stage("fvtp2d", {"q_i": o["q_i"], "q_j": o["q_j"], "fx1": o["fx1"], "fx2": o["fx2"], "fy1": o["fy1"],
                      "fy2": o["fy2"], "q": o["uout"], "crx": x["crx"], "cry": x["cry"], "ra_x": x["ra_x"],
                      "ra_y": x["ra_y"], "xfx": x["xfx"], "yfx": x["yfx"], "area": x["area"]},
           {"p1": s["ppm_p1"], "p2": s["ppm_p2"]}, nx, ny, nz, halo, 0)
    return o
