"""Batched ensembles: the chained step of uneven, mixed-precision members as persistent launches.

Every member's forward outputs and adjoint gradients from oeb_batch_run must be
bit-identical to the same member run alone through oeb_chain_forward_* / oeb_chain_adj_*
(the same kernels on the same tiles), after the autotuner has changed the k-blocking and
CTA counts, and when the run is replayed from a CUDA graph after the inputs change in place.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_bitwise_equal

pytestmark = pytest.mark.gpu

H = 8
SENTINEL = -7.0e5
# (nx, ny, nz, dtype): uneven, ragged tiles, both precisions
MEMBERS = [(48, 64, 7, np.float64), (80, 48, 5, np.float32), (64, 96, 9, np.float64), (33, 41, 3, np.float32),
           (17, 17, 2, np.float64), (128, 112, 12, np.float32), (1, 1, 1, np.float64)]


def _member(pkg, fields, chain, cuda, nx, ny, nz, dtype, seed):
    import torch
    x = fields.make_chain_inputs(nx, ny, nz, seed, halo=H)
    s = fields.make_chain_scalars(seed)
    shape = x["u"].shape

    def dev(a):
        a = np.ascontiguousarray(a, dtype=dtype)
        return pkg.Storage(torch.from_numpy(a).to(cuda), H, nx=nx if a.ndim == 3 else None)

    rng = np.random.default_rng([seed, 9])
    seeds = {}
    for n in chain.OUTPUTS:
        y = np.zeros(shape)
        y[H:H + nz, H:H + ny, H:H + nx] = rng.normal(0.0, 1.0, size=(nz, ny, nx))
        seeds[n] = dev(y)
    return {"fields": {k: dev(v) for k, v in x.items()}, "scalars": s, "domain": (nx, ny, nz),
            "outs": {n: dev(np.full(shape, SENTINEL)) for n in chain.OUTPUTS},
            "seeds": seeds, "grads": {n: dev(np.full(shape, SENTINEL)) for n in ("u", "v")},
            "dev": dev, "shape": shape}


def _alone(chain, m):
    """The member through its own chain plan, into fresh buffers."""
    import torch
    plan = chain.ChainPlan(m["fields"]["u"], m["domain"], chain.FORWARD | chain.ADJOINT)
    outs = {n: m["dev"](np.full(m["shape"], SENTINEL)) for n in chain.OUTPUTS}
    grads = {n: m["dev"](np.full(m["shape"], SENTINEL)) for n in ("u", "v")}
    plan.forward(m["fields"], m["scalars"], outs)
    plan.adjoint(m["fields"], m["scalars"], m["seeds"], grads)
    torch.cuda.synchronize()
    plan.close()
    return {n: v.numpy() for n, v in outs.items()}, {n: v.numpy() for n, v in grads.items()}


def _check(chain, members, what):
    for i, m in enumerate(members):
        outs, grads = _alone(chain, m)
        for n in chain.OUTPUTS:
            assert_bitwise_equal(m["outs"][n].numpy(), outs[n], "%s member %d %s" % (what, i, n))
        for n in ("u", "v"):
            assert_bitwise_equal(m["grads"][n].numpy(), grads[n], "%s member %d grad %s" % (what, i, n))


@pytest.fixture(scope="module")
def chain(pkg):
    import importlib
    return importlib.import_module("oeb_gb300.chain")


def test_batch_matches_members_run_alone(pkg, fields, chain, cuda):
    import torch
    members = [_member(pkg, fields, chain, cuda, nx, ny, nz, dt, 40 + i) for i, (nx, ny, nz, dt) in enumerate(MEMBERS)]
    plan = chain.BatchPlan(members, chain.FORWARD | chain.ADJOINT)
    assert plan.points == sum(nx * ny * nz for nx, ny, nz, _ in MEMBERS)
    lib = pkg.load_library()
    before = lib.oeb_launch_count()
    plan.run()
    torch.cuda.synchronize()
    assert lib.oeb_launch_count() - before == plan.launches
    _check(chain, members, "batch")
    # the autotuner changes k-blocking and CTA counts, not results
    plan.autotune()
    for m in members:
        for st in list(m["outs"].values()) + list(m["grads"].values()):
            st.data.fill_(SENTINEL)
    plan.run()
    torch.cuda.synchronize()
    _check(chain, members, "autotuned batch")
    plan.close()


def test_batch_graph_replay(pkg, fields, chain, cuda):
    import torch
    members = [_member(pkg, fields, chain, cuda, nx, ny, nz, dt, 60 + i)
               for i, (nx, ny, nz, dt) in enumerate(MEMBERS[:4])]
    plan = chain.BatchPlan(members, chain.FORWARD | chain.ADJOINT)
    stream = torch.cuda.Stream()
    plan.run(stream)  # one-time set-up outside the capture
    stream.synchronize()
    g = chain.Graph(stream)
    with g:
        plan.run(stream)
    for i, m in enumerate(members):  # new inputs in place
        nx, ny, nz = m["domain"]
        x2 = fields.make_chain_inputs(nx, ny, nz, 90 + i, halo=H)
        for k in ("u", "v", "utens", "mask", "crx"):
            m["fields"][k].data.copy_(torch.from_numpy(x2[k].astype(MEMBERS[i][3])).to(cuda))
        for st in list(m["outs"].values()) + list(m["grads"].values()):
            st.data.fill_(SENTINEL)
    torch.cuda.synchronize()
    g.launch(stream)
    stream.synchronize()
    _check(chain, members, "graph")
    g.close()
    plan.close()


def test_batch_rejects_a_member_without_outputs(pkg, fields, chain, cuda):
    m = _member(pkg, fields, chain, cuda, 16, 16, 2, np.float64, 7)
    del m["outs"]
    with pytest.raises(pkg.OebError):
        chain.BatchPlan([m], chain.FORWARD)


def _reset(members):
    for m in members:
        for st in list(m["outs"].values()) + list(m["grads"].values()):
            st.data.fill_(SENTINEL)


def test_tuning_record_applies_to_a_new_plan(pkg, fields, chain, cuda, tmp_path):
    # the autotuner's choices, saved by one plan and loaded by another over the same
    # ensemble, give the same launches and bit-identical results without timing anything
    import torch
    spec = MEMBERS[:5]

    def members():
        return [_member(pkg, fields, chain, cuda, nx, ny, nz, dt, 70 + i) for i, (nx, ny, nz, dt) in enumerate(spec)]

    a = chain.BatchPlan(members(), chain.FORWARD | chain.ADJOINT)
    default = a.tuning()
    assert default and all(c == (0, 0, 0) for c in default)
    a.autotune()
    tuned = a.tuning()
    # the autotuner may pick the fused grouping (hadvuv5th and the update as one kernel), which
    # records fewer launches
    assert a.fusion in (0, chain.FUSE_HADV_UPDATE)
    assert len(tuned) == len(default) if a.fusion == 0 else len(tuned) < len(default)
    assert all(kb in (1, 2, 4, 8) and shape in (0, 1, 2) and form in (0, 1, 2) for kb, shape, form in tuned)
    path = tmp_path / "tuning.json"
    a.save_tuning(path)
    b_members = members()
    b = chain.BatchPlan(b_members, chain.FORWARD | chain.ADJOINT)
    assert b.signature == a.signature
    b.load_tuning(path)
    assert b.tuning() == tuned
    assert b.launches == a.launches
    lib = pkg.load_library()
    before = lib.oeb_launch_count()
    b.run()
    torch.cuda.synchronize()
    assert lib.oeb_launch_count() - before == b.launches
    _check(chain, b_members, "tuning record applied")
    # the default choices as a record, in the default grouping, put the plan back
    b.set_fusion(0)
    b.apply_tuning(default)
    assert b.tuning() == default
    _reset(b_members)
    b.run()
    torch.cuda.synchronize()
    _check(chain, b_members, "default record applied")
    a.close()
    b.close()


def test_tuning_record_rejected_for_another_plan(pkg, fields, chain, cuda, tmp_path):
    # a record of another ensemble, of another format, or with a count, kb or form outside
    # the documented values is refused, and the plan keeps its choices
    a = chain.BatchPlan([_member(pkg, fields, chain, cuda, nx, ny, nz, dt, 80 + i)
                         for i, (nx, ny, nz, dt) in enumerate(MEMBERS[:2])], chain.FORWARD)
    path = tmp_path / "a.json"
    a.save_tuning(path)
    c = chain.BatchPlan([_member(pkg, fields, chain, cuda, nx, ny, nz, dt, 85 + i)
                         for i, (nx, ny, nz, dt) in enumerate(MEMBERS[1:3])], chain.FORWARD)
    assert c.signature != a.signature
    before = c.tuning()
    with pytest.raises(pkg.OebError):
        c.load_tuning(path)
    other = tmp_path / "other.json"
    other.write_text('{"format": "something-else", "signature": "%016x", "choices": []}' % c.signature)
    with pytest.raises(pkg.OebError):
        c.load_tuning(other)
    n = len(before)
    for bad in ([(0, 0, 0)] * (n + 1), [(3, 0, 0)] + before[1:], [(1, 0, 3)] + before[1:], [(-1, 0, 0)] + before[1:],
                [(1, 3, 0)] + before[1:], [(1, -1, 0)] + before[1:]):
        with pytest.raises(pkg.OebError) as err:
            c.apply_tuning(bad)
        assert err.value.status == 12  # OEB_ERR_ARGUMENT
    assert c.tuning() == before
    a.close()
    c.close()


# Members of benchmark configuration 5's sizes: nx, ny from {48..320} step 16, nz from
# {40, 60, 80, 137}, mixed precision; two of them 256 or more wide with 137 levels.
ORACLE_MEMBERS = [(272, 48, 137, np.float64), (48, 256, 137, np.float32), (64, 80, 40, np.float64),
                  (96, 48, 60, np.float32), (320, 64, 80, np.float64)]


def test_batch_members_match_the_oracle_step(pkg, fields, chain, cuda):
    # every FP64 member's forward outputs bit for bit against the step composed from the
    # oracle's stencils (oracle/chain.py); every FP32 member's normwise against that FP64 step,
    # both the total error and the error of the FP32 arithmetic alone (the FP64 step on the
    # FP32-rounded inputs)
    import torch
    from oracle import chain as ochain
    members = [_member(pkg, fields, chain, cuda, nx, ny, nz, dt, 140 + i)
               for i, (nx, ny, nz, dt) in enumerate(ORACLE_MEMBERS)]
    plan = chain.BatchPlan(members, chain.FORWARD | chain.ADJOINT)
    plan.autotune()
    for m in members:
        for st in list(m["outs"].values()) + list(m["grads"].values()):
            st.data.fill_(SENTINEL)
    plan.run()
    torch.cuda.synchronize()
    boxes = {"uout": 3, "vout": 3, "fx1": 0, "fy1": 0}
    for i, (m, (nx, ny, nz, dt)) in enumerate(zip(members, ORACLE_MEMBERS)):
        x = fields.make_chain_inputs(nx, ny, nz, 140 + i, halo=H)
        s = m["scalars"]

        def box(a, e):
            return a[H:H + nz, H - e:H + ny + e, H - e:H + nx + e]

        if dt == np.float64:
            want = ochain.run_chain(x, s, nx, ny, nz, H)
            for n in chain.OUTPUTS:
                assert_bitwise_equal(m["outs"][n].numpy(), want[n], "batched FP64 member %d (%dx%dx%d) %s" %
                                     (i, nx, ny, nz, n))
        else:
            want = ochain.run_chain(x, s, nx, ny, nz, H)
            xq = {k: v.astype(np.float32).astype(np.float64) for k, v in x.items()}
            sq = {k: float(np.float32(v)) for k, v in s.items()}
            want_q = ochain.run_chain(xq, sq, nx, ny, nz, H)
            for n, e in boxes.items():
                got = box(m["outs"][n].numpy().astype(np.float64), e)
                scale = float(np.max(np.abs(box(want[n], e))))
                tot = np.abs(got - box(want[n], e)) / scale
                ar = np.abs(got - box(want_q[n], e)) / scale
                what = "batched FP32 member %d (%dx%dx%d) %s" % (i, nx, ny, nz, n)
                # as the chained step alone: an fvtp2d limiter may flip where FP32 cannot
                # resolve the deciding difference
                assert int((ar > 1e-5).sum()) <= 1e-4 * ar.size + 2, what
                assert float(np.sqrt(np.mean(ar ** 2))) <= 1e-6, what
                assert float(np.sqrt(np.mean(tot ** 2))) <= 1e-5, what
    plan.close()
