"""The one-launch form of a batch plan: every member's chained step, forward then adjoint, FP64
and FP32 members alike, in ONE persistent launch of the step kernel.

* Results are bit-identical to each member run alone through its chain plan (and so to the
  per-launch form, which the oracle pins), with each kernel's default k-blocking and another,
  after the form autotuner, and when the run is replayed from a CUDA graph.
* A run is one kernel launch.
* The waits are bounded: a task made to wait for a count that nothing writes ends the run with
  OEB_ERR_TIMEOUT after a short limit -- no fault, no hang -- and the next run is correct.
* Members of the ensemble benchmark's sizes (up to 320 wide, 137 levels) match the per-launch
  form bit for bit.
"""
from __future__ import annotations

import time

import numpy as np
import pytest

from conftest import assert_bitwise_equal
from test_gpu_batch import MEMBERS, ORACLE_MEMBERS, H, _check, _member, _reset

pytestmark = pytest.mark.gpu

OEB_ERR_TIMEOUT = 10


@pytest.fixture(scope="module")
def chain(pkg):
    import importlib
    return importlib.import_module("oeb_gb300.chain")


def test_one_launch_matches_members_run_alone(pkg, fields, chain, cuda):
    import torch
    members = [_member(pkg, fields, chain, cuda, nx, ny, nz, dt, 240 + i)
               for i, (nx, ny, nz, dt) in enumerate(MEMBERS)]
    plan = chain.BatchPlan(members, chain.FORWARD | chain.ADJOINT)
    lib = pkg.load_library()
    assert plan.form == (plan.PER_LAUNCH, -1, -1)
    for kb, per_sm in ((0, 2), (2, 3), (1, 4)):
        plan.set_form(plan.ONE_LAUNCH, kb, per_sm)
        assert plan.form == (plan.ONE_LAUNCH, kb, per_sm)
        assert plan.launches == 1
        _reset(members)
        before = lib.oeb_launch_count()
        plan.run()
        torch.cuda.synchronize()
        assert lib.oeb_launch_count() - before == 1
        assert plan.step_status() == (0, -1)
        _check(chain, members, "one launch, kb %d, %d CTAs an SM" % (kb, per_sm))
    with pytest.raises(pkg.OebError):
        plan.set_form(plan.ONE_LAUNCH, 3, 2)  # kb not one the recordings take
    with pytest.raises(pkg.OebError):
        plan.set_form(plan.ONE_LAUNCH, 0, 5)  # no such build
    # the form autotuner picks a form and a k-blocking; results do not change
    ms = plan.autotune_form()
    assert ms > 0.0
    _reset(members)
    plan.run()
    torch.cuda.synchronize()
    assert plan.step_status() == (0, -1)
    _check(chain, members, "autotuned form %s" % (plan.form,))
    plan.close()


def test_one_launch_wait_limit_and_graph(pkg, fields, chain, cuda):
    import torch
    members = [_member(pkg, fields, chain, cuda, nx, ny, nz, dt, 260 + i)
               for i, (nx, ny, nz, dt) in enumerate(MEMBERS[:4])]
    plan = chain.BatchPlan(members, chain.FORWARD | chain.ADJOINT)
    with pytest.raises(pkg.OebError):
        plan.withhold(True)  # no one-launch tables yet
    plan.set_form(plan.ONE_LAUNCH, 0)
    # the first task waits for a count that nothing writes: past the 2 ms limit its CTA gives
    # up, every other CTA stops at its next tile, and the status says so
    plan.set_wait_limit(2_000_000)
    plan.withhold(True)
    t0 = time.time()
    plan.run()
    torch.cuda.synchronize()
    elapsed = time.time() - t0
    status, task = plan.step_status()
    assert status == OEB_ERR_TIMEOUT and task >= 0, (status, task)
    assert elapsed < 10.0
    # restored, the plan runs correctly, also as a CUDA graph with new inputs in place
    plan.withhold(False)
    plan.set_wait_limit(2_000_000_000)
    stream = torch.cuda.Stream()
    g = chain.Graph(stream)
    with g:
        plan.run(stream)
    for i, m in enumerate(members):
        nx, ny, nz = m["domain"]
        x2 = fields.make_chain_inputs(nx, ny, nz, 290 + i, halo=H)
        for k in ("u", "v", "utens", "mask", "crx"):
            m["fields"][k].data.copy_(torch.from_numpy(x2[k].astype(MEMBERS[i][3])).to(cuda))
    _reset(members)
    torch.cuda.synchronize()
    g.launch(stream)
    stream.synchronize()
    assert plan.step_status() == (0, -1)
    _check(chain, members, "one launch from a graph")
    g.close()
    plan.close()


def test_one_launch_matches_per_launch_form_at_ensemble_sizes(pkg, fields, chain, cuda):
    # members of the ensemble benchmark's sizes (two 256 or more wide with 137 levels), mixed
    # precision: the one-launch form against the per-launch form, whose members the oracle
    # step pins (test_gpu_batch.py)
    import torch
    members = [_member(pkg, fields, chain, cuda, nx, ny, nz, dt, 340 + i)
               for i, (nx, ny, nz, dt) in enumerate(ORACLE_MEMBERS)]
    plan = chain.BatchPlan(members, chain.FORWARD | chain.ADJOINT)
    plan.run()
    torch.cuda.synchronize()
    want = [({n: v.numpy() for n, v in m["outs"].items()}, {n: v.numpy() for n, v in m["grads"].items()})
            for m in members]
    for kb, per_sm in ((0, 2), (4, 3)):
        plan.set_form(plan.ONE_LAUNCH, kb, per_sm)
        _reset(members)
        plan.run()
        torch.cuda.synchronize()
        assert plan.step_status() == (0, -1)
        for i, (m, (outs, grads)) in enumerate(zip(members, want)):
            for n in chain.OUTPUTS:
                assert_bitwise_equal(m["outs"][n].numpy(), outs[n], "kb %d member %d %s" % (kb, i, n))
            for n in ("u", "v"):
                assert_bitwise_equal(m["grads"][n].numpy(), grads[n], "kb %d member %d grad %s" % (kb, i, n))
    plan.close()
