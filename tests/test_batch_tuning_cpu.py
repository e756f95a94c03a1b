"""Batch tuning records without a GPU: the C ABI's NULL checks, and the Python side of
BatchPlan.save_tuning / load_tuning (file format, signature check, hand-over of the choices).

The native plan calls are replaced by a stand-in subclass, so only the host logic runs here;
tests/test_gpu_batch.py applies real records to real plans.
"""
from __future__ import annotations

import ctypes
import importlib
import json

import pytest


@pytest.fixture(scope="module")
def chain(pkg):
    return importlib.import_module("oeb_gb300.chain")


def _stand_in(chain, signature, choices, fusion=0):
    class Plan(chain.BatchPlan):
        def __init__(self):
            self._plan = ctypes.c_void_p()
            self.applied = None
            self._fusion = fusion

        @property
        def signature(self):
            return signature

        @property
        def fusion(self):
            return self._fusion

        def set_fusion(self, mask):
            self._fusion = mask

        def tuning(self):
            return list(choices)

        def apply_tuning(self, rec):
            self.applied = [tuple(c) for c in rec]

        def close(self):
            pass

    return Plan()


def test_abi_rejects_a_null_plan(pkg):
    lib = pkg.load_library()
    n = ctypes.c_int(-1)
    sig = ctypes.c_uint64()
    rec = (ctypes.c_int * 6)()
    assert lib.oeb_batch_tuning_get(None, rec, 2, ctypes.byref(n)) == 1  # OEB_ERR_NULL
    assert lib.oeb_batch_tuning_apply(None, rec, 2) == 1
    assert lib.oeb_batch_signature(None, ctypes.byref(sig)) == 1
    # the one-launch form's entry points
    form, kb, st = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert lib.oeb_batch_set_form(None, 1, 0, 2) == 1
    assert lib.oeb_batch_get_form(None, ctypes.byref(form), ctypes.byref(kb), ctypes.byref(st)) == 1
    us, n = ctypes.c_uint64(), ctypes.c_uint64()
    assert lib.oeb_batch_step_waits(None, ctypes.byref(us), ctypes.byref(n)) == 1
    assert lib.oeb_batch_autotune_form(None, None, None) == 1
    assert lib.oeb_batch_step_status(None, ctypes.byref(st), None) == 1
    assert lib.oeb_batch_set_wait_limit(None, ctypes.c_uint64(1000)) == 1
    assert lib.oeb_batch_withhold(None, 1) == 1
    mask = ctypes.c_int()
    assert lib.oeb_batch_set_fusion(None, 1) == 1
    assert lib.oeb_batch_get_fusion(None, ctypes.byref(mask)) == 1
    assert lib.oeb_set_fusion(2) == 12  # OEB_ERR_ARGUMENT: no such grouping
    assert lib.oeb_set_fusion(0) == 0
    assert lib.oeb_set_adjoint_tiles(2) == 12  # OEB_ERR_ARGUMENT: 0 or 1
    assert lib.oeb_set_adjoint_tiles(1) == 0


def test_saved_record_is_applied_to_a_plan_with_the_same_signature(chain, tmp_path):
    choices = [(4, 0, 0), (1, 2, 2), (8, 1, 1), (0, 0, 0)]
    a = _stand_in(chain, 0x0123456789ABCDEF, choices, fusion=chain.FUSE_HADV_UPDATE)
    path = tmp_path / "t.json"
    a.save_tuning(path)
    rec = json.loads(path.read_text())
    assert rec == {"format": chain.BatchPlan.TUNING_FORMAT, "signature": "0123456789abcdef",
                   "fusion": chain.FUSE_HADV_UPDATE, "choices": [list(c) for c in choices]}
    # the record's fusion grouping is set before its choices are applied
    b = _stand_in(chain, 0x0123456789ABCDEF, [(0, 0, 0)] * 5)
    b.load_tuning(path)
    assert b.fusion == chain.FUSE_HADV_UPDATE
    assert b.applied == choices


def test_record_of_another_ensemble_or_format_is_refused(pkg, chain, tmp_path):
    path = tmp_path / "t.json"
    _stand_in(chain, 7, [(2, 1, 0)]).save_tuning(path)
    other = _stand_in(chain, 8, [(0, 0, 0)])
    with pytest.raises(pkg.OebError, match="another ensemble"):
        other.load_tuning(path)
    assert other.applied is None
    rec = json.loads(path.read_text())
    rec["format"] = "oeb-batch-tuning/1"
    path.write_text(json.dumps(rec))
    same = _stand_in(chain, 7, [(0, 0, 0)])
    with pytest.raises(pkg.OebError, match="not a batch tuning record"):
        same.load_tuning(path)
    assert same.applied is None


def test_one_launch_ticket_order_keeps_every_member_in_order(pkg):
    # The step kernel's waits end because a task waits only for its member's previous task,
    # which always holds an earlier ticket: checked on the plan's own ordering function over
    # random uneven ensembles, then by playing the tickets through a few CTAs that each wait
    # only for what earlier tickets complete.
    import numpy as np
    lib = pkg.load_library()
    rng = np.random.default_rng(12)
    for trial in range(40):
        m = int(rng.integers(1, 60))
        counts = rng.integers(0 if trial % 5 == 0 else 1, 40, size=m).astype(np.int32)
        points = rng.integers(1, 1 << 24, size=m).astype(np.int64)
        if trial % 7 == 0:
            points[:] = 1000  # ties everywhere
        n = int(counts.sum())
        member = np.full(max(n, 1), -9, np.int32)
        pos = np.full(max(n, 1), -9, np.int32)
        dep = np.full(max(n, 1), -9, np.int32)
        p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        assert lib.oeb_batch_step_order(ctypes.c_int(m), p(counts), p(points), p(member), p(pos), p(dep)) == 0
        seen = {}
        for t in range(n):
            mb, q = int(member[t]), int(pos[t])
            assert 0 <= mb < m and q == seen.get(mb, 0), (trial, t, mb, q)  # each member in order
            seen[mb] = q + 1
            if q == 0:
                assert dep[t] == -1
            else:
                d = int(dep[t])
                assert 0 <= d < t and member[d] == mb and pos[d] == q - 1, (trial, t)
        assert all(seen.get(i, 0) == counts[i] for i in range(m))
        # a few CTAs take tickets in order; a CTA holding ticket t runs once dep[t] is done
        done = np.zeros(max(n, 1), bool)
        ctas = int(rng.integers(1, 9))
        next_ticket, held = 0, []
        for _ in range(4 * n + 10):
            while len(held) < ctas and next_ticket < n:
                held.append(next_ticket)
                next_ticket += 1
            runnable = [t for t in held if dep[t] < 0 or done[dep[t]]]
            if not runnable:
                break
            done[runnable[0]] = True
            held.remove(runnable[0])
        assert next_ticket == n and not held, "tickets left waiting: %d of %d" % (n - int(done.sum()), n)
    # argument checks
    one = np.ones(1, np.int32)
    pts = np.ones(1, np.int64)
    out = np.zeros(1, np.int32)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert lib.oeb_batch_step_order(0, p(one), p(pts), p(out), p(out), p(out)) == 12
    assert lib.oeb_batch_step_order(1, None, p(pts), p(out), p(out), p(out)) == 1
    neg = np.full(1, -1, np.int32)
    assert lib.oeb_batch_step_order(1, p(neg), p(pts), p(out), p(out), p(out)) == 12
