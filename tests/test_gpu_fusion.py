"""Fusion groupings of the chained step (oeb_set_fusion, oeb_batch_set_fusion).

OEB_FUSE_HADV_UPDATE runs hadvuv5th and the explicit update as one kernel, and in the adjoint
step the hadvuv5th gather and the update's transpose as one kernel.  The fused step must give
the unfused step's results bit for bit -- FP64 and FP32, forward and adjoint, at several sizes
-- with fewer launches; batch plans in either grouping, in the per-launch and the one-launch
form, must match members run alone; the autotuner's grouping travels in a tuning record.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import assert_bitwise_equal
from test_gpu_batch import MEMBERS, SENTINEL, _check, _member, _reset
from test_gpu_chain import Step

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def chain(pkg):
    import importlib
    return importlib.import_module("oeb_gb300.chain")


def _set_fusion(pkg, mask):
    assert pkg.load_library().oeb_set_fusion(ctypes.c_int(mask)) == 0


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("size", [(128, 128, 80), (37, 45, 5), (1, 1, 1)])
def test_fused_step_matches_unfused(pkg, fields, chain, cuda, size, dtype):
    nx, ny, nz = size
    st = Step(pkg, fields, chain, cuda, nx, ny, nz, 23, chain.FORWARD | chain.ADJOINT, dtype=dtype)
    rng = np.random.default_rng(5)
    seeds = {}
    for n in chain.OUTPUTS:
        y = np.zeros(st.shape)
        y[8:8 + nz, 8:8 + ny, 8:8 + nx] = rng.normal(size=(nz, ny, nx))
        seeds[n] = y
    lib = pkg.load_library()
    runs = {}
    try:
        for mask in (0, chain.FUSE_HADV_UPDATE):
            _set_fusion(pkg, mask)
            l0 = lib.oeb_launch_count()
            fwd = st.forward()
            l1 = lib.oeb_launch_count()
            adj = st.adj(seeds)
            l2 = lib.oeb_launch_count()
            runs[mask] = (fwd, adj, l1 - l0, l2 - l1)
    finally:
        _set_fusion(pkg, chain.FUSE_HADV_UPDATE)  # the default
    (f0, a0, lf0, la0), (f1, a1, lf1, la1) = runs[0], runs[chain.FUSE_HADV_UPDATE]
    for n in chain.OUTPUTS:
        assert_bitwise_equal(f1[n], f0[n], "fused forward %s" % n)
    for n in ("u", "v"):
        assert_bitwise_equal(a1[n], a0[n], "fused adjoint grad %s" % n)
    # two update launches fewer in the forward step, four in the adjoint step (its recompute
    # of the forward stages and the update's transpose)
    assert lf1 == lf0 - 2 and la1 == la0 - 4, (lf0, lf1, la0, la1)


def test_batch_fusion_groupings_match_members_alone(pkg, fields, chain, cuda):
    import torch
    members = [_member(pkg, fields, chain, cuda, nx, ny, nz, dt, 400 + i) for i, (nx, ny, nz, dt) in enumerate(MEMBERS)]
    plan = chain.BatchPlan(members, chain.FORWARD | chain.ADJOINT)
    assert plan.fusion == 0
    sig = plan.signature
    base = plan.launches
    plan.set_fusion(chain.FUSE_HADV_UPDATE)
    assert plan.fusion == chain.FUSE_HADV_UPDATE
    assert plan.signature == sig  # a grouping does not change which ensemble the plan is
    assert plan.launches < base
    _reset(members)
    plan.run()
    torch.cuda.synchronize()
    _check(chain, members, "fused batch")
    plan.set_form(plan.ONE_LAUNCH, 2, 4)
    _reset(members)
    plan.run()
    torch.cuda.synchronize()
    assert plan.step_status() == (0, -1)
    _check(chain, members, "fused batch, one launch")
    # back to the unfused grouping: the one-launch tables follow
    plan.set_fusion(0)
    _reset(members)
    plan.run()
    torch.cuda.synchronize()
    _check(chain, members, "unfused batch, one launch")
    with pytest.raises(pkg.OebError):
        plan.set_fusion(2)
    plan.close()


def test_autotuned_grouping_travels_in_the_tuning_record(pkg, fields, chain, cuda, tmp_path):
    import torch
    spec = MEMBERS[:5]
    members = [_member(pkg, fields, chain, cuda, nx, ny, nz, dt, 420 + i) for i, (nx, ny, nz, dt) in enumerate(spec)]
    a = chain.BatchPlan(members, chain.FORWARD | chain.ADJOINT)
    a.autotune()
    path = tmp_path / "rec.json"
    a.save_tuning(path)
    b = chain.BatchPlan(members, chain.FORWARD | chain.ADJOINT)
    b.load_tuning(path)
    assert b.fusion == a.fusion
    assert b.tuning() == a.tuning()
    assert b.launches == a.launches
    _reset(members)
    b.run()
    torch.cuda.synchronize()
    _check(chain, members, "batch from a tuning record")
    a.close()
    b.close()
