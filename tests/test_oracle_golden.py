"""The oracle against the golden vectors made by the reference itself (tests/golden/).

The vectors are outputs of the reference's own kernels compiled from its source tree
(tests/golden/make_golden.py); the reference has no tests or fixtures of its own.  The oracle
must reproduce every output cell bit for bit (cells outside each written box included),
in FP64 and FP32.  These tests need no GPU and no reference source tree.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from conftest import assert_bitwise_equal

GOLDEN = Path(__file__).resolve().parent / "golden"
KERNELS = ("laplace", "hdiffsa", "hdiffsmag", "hadvuv", "hadvuv5th", "fastwavesuv", "uvbke", "nh_p_grad",
           "p_grad_c", "fvtp2d")


def _case(data, case):
    meta = json.loads(str(data["%s/meta" % case]))
    scalars = json.loads(str(data["%s/scalars" % case]))
    fields = {k.split("/", 1)[1]: data[k] for k in data.files if k.startswith(case + "/")
              and not k.endswith(("/meta", "/scalars"))}
    return meta, scalars, fields


@pytest.mark.parametrize("case", ("driver", "physical", "physical_f32"))
@pytest.mark.parametrize("name", KERNELS)
def test_oracle_matches_reference_golden(pkg, orc, name, case):
    spec = pkg.KERNELS[name]
    data = np.load(GOLDEN / ("%s.npz" % name))
    meta, scalars, golden = _case(data, case)
    n, nz, h = meta["n"], meta["nz"], meta["halo"]
    dtype = np.dtype(meta["dtype"])
    bufs = {}
    for a in spec.args:
        if a.role in ("in3", "in1"):
            bufs[a.name] = golden[a.name].copy()
        elif a.role == "out3":
            # outputs start from what the reference call started from: the golden value
            # outside the written box (the reference leaves those cells untouched)
            bufs[a.name] = np.full_like(golden[a.name], np.nan)
    # the written boxes: fill everything outside from the golden vector, inside with NaN
    for a in spec.by_role("out3"):
        ilo, ihi, jlo, jhi, klo, khi = a.reach
        g = golden[a.name]
        b = bufs[a.name]
        b[...] = g
        b[h - klo:h + nz + khi, h - jlo:h + n + jhi, h - ilo:h + n + ihi] = np.nan
    orc.run_oracle(spec, bufs, scalars, n, n, nz, h)
    assert all(bufs[a.name].dtype == dtype for a in spec.by_role("out3"))
    for a in spec.by_role("out3"):
        assert_bitwise_equal(bufs[a.name], golden[a.name], "%s/%s.%s" % (name, case, a.name))


def test_golden_cases_exercise_the_branches(pkg):
    """The physical golden inputs make the data-dependent branches go both ways."""
    data = np.load(GOLDEN / "fvtp2d.npz")
    _, _, g = _case(data, "physical")
    assert (g["crx"] > 0).any() and (g["crx"] <= 0).any()
    assert (g["q"] > 0).any() and (g["q"] < 0).any()
    data = np.load(GOLDEN / "hadvuv5th.npz")
    _, _, g = _case(data, "physical")
    assert (g["uin"] > 0).any() and (g["uin"] < 0).any()
