"""The FP32 adjoints in one tiled launch (oeb_set_adjoint_tiles(1), the default) against their
multi-pass forms (terms or coefficients in scratch, oeb_set_adjoint_tiles(0)): hdiffsmag,
hadvuv, hadvuv5th, fastwavesuv, p_grad_c and nh_p_grad.  The tiled kernels form the same terms with the same
expressions and gather them in the same order, so every gradient cell -- inside and outside
the written boxes -- must be the same bits, at the benchmark size, on ragged domains whose
tiles are cut at every edge, and on a single cell.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import assert_bitwise_equal
from test_gpu_adjoint import Case

pytestmark = pytest.mark.gpu

TILED = ("hdiffsmag", "hadvuv", "hadvuv5th", "fastwavesuv", "p_grad_c", "nh_p_grad")


@pytest.mark.parametrize("name", TILED)
@pytest.mark.parametrize("size", [(128, 128, 80), (70, 97, 9), (33, 31, 3), (1, 1, 1), (40, 17, 30)],
                         ids=["128x128x80", "70x97x9", "33x31x3", "1x1x1", "40x17x30"])
def test_tiled_fp32_adjoint_matches_multipass(pkg, fields, cuda, name, size):
    nx, ny, nz = size
    case = Case(pkg, fields, cuda, name, nx, ny, nz, seed=17, workload="fronts", dtype=np.float32)
    rng = np.random.default_rng(5)
    ybar = {n: rng.normal(size=case.shape3()) for n in case.spec.semantic_outputs}
    lib = pkg.load_library()
    got = {}
    try:
        for tiles in (1, 0):
            assert lib.oeb_set_adjoint_tiles(ctypes.c_int(tiles)) == 0
            got[tiles] = case.adj(ybar)
    finally:
        lib.oeb_set_adjoint_tiles(ctypes.c_int(1))
    for n in case.active:
        assert_bitwise_equal(got[1][n].astype(np.float32), got[0][n].astype(np.float32),
                             "%s %dx%dx%d: tiled vs multi-pass %sb" % (name, nx, ny, nz, n))

