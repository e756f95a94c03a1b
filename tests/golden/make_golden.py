#!/usr/bin/env python3
"""Generates tests/golden/<kernel>.npz from the reference itself.

The reference ships no tests, fixtures or known-answer vectors, so the golden vectors are
outputs of the reference's own kernels (kernels/*.h) compiled from its source tree into
oracle/_ref/liboeb_ref.so by oracle/build.py.  Two cases per kernel, both on a square
6 x 6 interior (the reference's domain is square):

* ``driver``   -- the reference drivers' own inputs: fillMath with the parameters of
                  src/<k>.cpp, run through the reference's own fillMath/initValue
                  (include/util.h:150-196), halo 4 (src/<k>.cpp:6), the drivers' scalars and
                  output initial values.  fillMath leaves the k-halo planes unset
                  (util.h:159); here every cell is zeroed first, so those planes read 0.
                  Kernel: the `_openmp` variant (serial fvtp2d).  nz = 3.
* ``physical`` -- seeded inputs from fields.py (halo 3, nz = 2), in FP64 and FP32.

Each file stores, under "<case>/<field>", every input and the outputs after the call, plus
"<case>/scalars" (JSON) and "<case>/meta" (JSON: n, nz, halo, dtype).
Run: python tests/golden/make_golden.py   (needs the reference source tree)
"""
from __future__ import annotations

import ctypes
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import __graft_entry__ as graft  # noqa: E402

# fillMath parameters of every field in the drivers (src/<k>.cpp), and output initial values.
DRIVER_FILL = {
    "laplace": {"in": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1)},
    "hdiffsa": {"in": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1), "crlato": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5),
                "crlatu": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5), "mask": 0.025},
    "hdiffsmag": {"uin": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1), "vin": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5),
                  "crlavo": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5), "crlavu": (5.0, 8.0, 1.5, 7.1, 2.0, 4.3),
                  "crlato": (5.0, 8.0, 1.5, 7.1, 2.0, 4.3), "crlatu": (3.2, 7.0, 2.5, 6.1, 3.0, 2.3),
                  "acrlat0": (4.5, 5.0, 2.5, 2.1, 3.0, 2.3), "mask": 0.025},
    "hadvuv": {"uin": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1), "vin": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5),
               "acrlat0": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5), "acrlat1": (5.0, 8.0, 1.5, 7.1, 2.0, 4.3),
               "tgrlatda0": (5.0, 8.0, 1.5, 7.1, 2.0, 4.3), "tgrlatda1": (3.2, 7.0, 2.5, 6.1, 3.0, 2.3)},
    "hadvuv5th": {"uin": (1.0, 3.3, 1.5, 1.5, 2.0, 4.0), "vin": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1),
                  "acrlat0": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1), "acrlat1": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5),
                  "tgrlatda0": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5), "tgrlatda1": (5.0, 8.0, 1.5, 7.1, 2.0, 4.3)},
    "fastwavesuv": {"uin": (1.0, 3.3, 1.5, 1.5, 2.0, 4.0), "utens": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1),
                    "vin": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1), "vtens": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5),
                    "ppuv": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5), "wgtfac": (5.0, 8.0, 1.5, 7.1, 2.0, 4.3),
                    "hhl": (5.0, 8.0, 1.5, 7.1, 2.0, 4.3), "rho": (3.2, 7.0, 2.5, 6.1, 3.0, 2.3),
                    "fx": (4.5, 5.0, 2.5, 2.1, 3.0, 2.3)},
    "uvbke": {"uc": (1.0, 3.3, 1.5, 1.5, 2.0, 4.0), "vc": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1),
              "cosa": (4.0, 1.7, 1.5, 6.3, 2.0, 1.4), "rsina": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5)},
    "nh_p_grad": {"uin": (1.0, 3.3, 1.5, 1.5, 2.0, 4.0), "vin": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1),
                  "rdx": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1), "rdy": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5),
                  "gz": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5), "pp": (5.0, 8.0, 1.5, 7.1, 2.0, 4.3),
                  "pk3": (5.0, 8.0, 1.5, 7.1, 2.0, 4.3), "wk1": (3.2, 7.0, 2.5, 6.1, 3.0, 2.3)},
    "p_grad_c": {"uin": (1.0, 3.3, 1.5, 1.5, 2.0, 4.0), "vin": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1),
                 "rdxc": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1), "rdyc": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5),
                 "delpc": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5), "gz": (5.0, 8.0, 1.5, 7.1, 2.0, 4.3),
                 "pkc": (5.0, 8.0, 1.5, 7.1, 2.0, 4.3)},
    "fvtp2d": {"q": (1.0, 3.3, 1.5, 1.5, 2.0, 4.0), "crx": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1),
               "cry": (1.1, 2.0, 1.5, 2.8, 2.0, 4.1), "ra_x": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5),
               "ra_y": (8.0, 9.4, 1.5, 1.7, 2.0, 3.5), "xfx": (5.0, 8.0, 1.5, 7.1, 2.0, 4.3),
               "yfx": (5.0, 8.0, 1.5, 7.1, 2.0, 4.3), "area": (3.2, 7.0, 2.5, 6.1, 3.0, 2.3)},
}
# initValue of the outputs in the drivers (src/uvbke.cpp:51-52, src/fvtp2d.cpp:71-76; 0.0 elsewhere)
OUT_INIT = {"uvbke": -1.0, "fvtp2d": -1.0}

N, NZ_DRIVER, HALO_DRIVER = 6, 3, 4
NZ_PHYS, HALO_PHYS, SEED_PHYS = 2, 3, 21


def driver_case(pkg, orc, name):
    spec = pkg.KERNELS[name]
    lib = orc._lib("ref")
    n, nz, h = N, NZ_DRIVER, HALO_DRIVER
    shape3 = (nz + 2 * h, n + 2 * h, n + 2 * h)
    bufs = {}
    for a in spec.args:
        if a.role == "in1":
            arr = np.zeros(n + 2 * h)
            m = orc.memref(arr, h)
            lib.oeb_ref_fillmath1_f64(*map(ctypes.c_double, DRIVER_FILL[name][a.name]), ctypes.byref(m),
                                      ctypes.c_int64(n), ctypes.c_int64(nz), ctypes.c_int64(h))
            bufs[a.name] = arr
        elif a.role in ("in3", "out3"):
            arr = np.zeros(shape3)
            m = orc.memref(arr, h)
            fill = DRIVER_FILL[name].get(a.name) if a.role == "in3" else OUT_INIT.get(name, 0.0)
            if isinstance(fill, tuple):
                lib.oeb_ref_fillmath3_f64(*map(ctypes.c_double, fill), ctypes.byref(m), ctypes.c_int64(n),
                                          ctypes.c_int64(nz), ctypes.c_int64(h))
            else:
                lib.oeb_ref_initvalue3_f64(ctypes.byref(m), ctypes.c_double(fill), ctypes.c_int64(n),
                                           ctypes.c_int64(nz), ctypes.c_int64(h))
            bufs[a.name] = arr
    inputs = {k: v.copy() for k, v in bufs.items()}
    scalars = dict(pkg.DRIVER_SCALARS.get(name, {}))
    orc.run_reference(spec, bufs, scalars, n, nz, h, "openmp")
    return inputs, bufs, scalars, {"n": n, "nz": nz, "halo": h, "dtype": "float64"}


def physical_case(pkg, orc, fields, name, dtype):
    spec = pkg.KERNELS[name]
    n, nz, h = N, NZ_PHYS, HALO_PHYS
    inputs = fields.make_inputs(name, n, n, nz, seed=SEED_PHYS, halo=h, dtype=dtype)
    outs = fields.make_outputs(name, n, n, nz, halo=h, dtype=dtype)
    bufs = {k: v.copy() for k, v in {**inputs, **outs}.items()}
    scalars = fields.make_scalars(name, seed=SEED_PHYS)
    if dtype == np.float32:  # the scalars the FP32 reference sees are ElementType values
        scalars = {k: (v if s.always_double else float(np.float32(v)))
                   for (k, v), s in zip(scalars.items(), spec.scalars)}
    orc.run_reference(spec, bufs, scalars, n, nz, h, "openmp")
    return inputs, bufs, scalars, {"n": n, "nz": nz, "halo": h, "dtype": np.dtype(dtype).name}


def main():
    graft.build()
    pkg = graft.load_package()
    import importlib
    fields = importlib.import_module("oeb_gb300.fields")
    from oracle import oracle as orc
    if not orc.reference_available():
        sys.exit("the reference source tree is needed to make golden vectors")
    out_dir = Path(__file__).resolve().parent
    for name, spec in pkg.KERNELS.items():
        data = {}
        cases = [("driver", driver_case(pkg, orc, name)),
                 ("physical", physical_case(pkg, orc, fields, name, np.float64)),
                 ("physical_f32", physical_case(pkg, orc, fields, name, np.float32))]
        for case, (inputs, bufs, scalars, meta) in cases:
            for a in spec.args:
                if a.role in ("in3", "in1"):
                    data["%s/%s" % (case, a.name)] = inputs[a.name]
                elif a.role == "out3":
                    data["%s/%s" % (case, a.name)] = bufs[a.name]
            data["%s/scalars" % case] = np.array(json.dumps(scalars))
            data["%s/meta" % case] = np.array(json.dumps(meta))
        np.savez_compressed(out_dir / ("%s.npz" % name), **data)
        print("wrote", name)


if __name__ == "__main__":
    main()
