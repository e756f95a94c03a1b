"""oeb_hdiffsmag_adj_noalloc_f64: the hdiffsmag adjoint on the library's fixed scratch array.

The entry point exists for callers that cannot allocate device memory while they run. One
example is a host whose own allocator reserved the GPU's memory at start-up, where a pool
allocation could fail mid-run; another is a time-step loop that must not allocate in its step.

It must give the same results as the pool-backed oeb_hdiffsmag_adj_f64 (bit for bit: the
same kernels on the same arguments), on consecutive calls that reuse the array with
different sizes, and reject fields whose allocation exceeds the array (2^21 cells) before
anything runs.  Both entry points are called through the C ABI.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import assert_bitwise_equal

H = 3
CAPACITY_CELLS = 1 << 21
SENTINEL = -7.0e5
OEB_ERR_TOO_LARGE = 11


def _args(pkg, st, xb, yb, sc, dom):
    names3 = ("uin", "vin", "mask")
    names1 = ("crlavo", "crlavu", "crlato", "crlatu", "acrlat0")
    refs = [ctypes.byref(xb["uin"].memref()), ctypes.byref(xb["vin"].memref())]
    refs += [ctypes.byref(st[n].memref()) for n in names3 + names1]
    refs += [ctypes.byref(yb["uout"].memref()), ctypes.byref(yb["vout"].memref())]
    refs += [ctypes.c_double(sc[n]) for n in ("eddlat", "eddlon", "tau_smag", "weight_smag")]
    return refs + [ctypes.byref(pkg.Domain(*dom)), ctypes.c_void_p(0)]


def _call(pkg, name, args):
    fn = getattr(pkg.load_library(), name)
    fn.restype = ctypes.c_int
    return fn(*args)


def _case(pkg, fields, cuda, nx, ny, nz, seed, workload):
    import torch
    x = fields.make_inputs("hdiffsmag", nx, ny, nz, seed=seed, workload=workload, halo=H)
    sc = fields.make_scalars("hdiffsmag", seed=seed)
    rng = np.random.default_rng([seed, 5])
    shape = (nz + 2 * H, ny + 2 * H, nx + 2 * H)

    def dev(a):
        return pkg.Storage(torch.from_numpy(np.ascontiguousarray(a)).to(cuda), H, nx=nx if a.ndim == 3 else None)

    st = {k: dev(v) for k, v in x.items()}
    yb = {n: dev(rng.normal(0.0, 1.0, size=shape)) for n in ("uout", "vout")}
    return st, yb, sc, shape, dev


@pytest.mark.gpu
def test_noalloc_adjoint_matches_pool_adjoint_on_consecutive_calls(pkg, fields, cuda):
    import torch
    cases = [(128, 128, 80, 3, "physical"), (70, 97, 9, 5, "fronts"), (40, 36, 5, 6, "physical")]
    for nx, ny, nz, seed, workload in cases:
        st, yb, sc, shape, dev = _case(pkg, fields, cuda, nx, ny, nz, seed, workload)
        want = {n: dev(np.full(shape, SENTINEL)) for n in ("uin", "vin")}
        got = {n: dev(np.full(shape, SENTINEL)) for n in ("uin", "vin")}
        dom = (nx, ny, nz)
        assert _call(pkg, "oeb_hdiffsmag_adj_f64", _args(pkg, st, want, yb, sc, dom)) == 0
        # twice in a row: the second call starts from the first call's array contents
        for _ in range(2):
            got["uin"].data.fill_(SENTINEL)
            got["vin"].data.fill_(SENTINEL)
            status = _call(pkg, "oeb_hdiffsmag_adj_noalloc_f64", _args(pkg, st, got, yb, sc, dom))
            assert status == 0, pkg.load_library().oeb_status_string(status)
            torch.cuda.synchronize()
            for n in ("uin", "vin"):
                assert_bitwise_equal(got[n].numpy(), want[n].numpy(), "%s bar %s" % (n, dom))


def test_noalloc_adjoint_rejects_fields_beyond_its_capacity(pkg):
    # 166 x 166 x 86 cells = 2,369,816 > 2^21: rejected by the checks, before any CUDA call
    nx = ny = 160
    nz = 80
    shape = (nz + 2 * H, ny + 2 * H, nx + 2 * H)
    assert shape[0] * shape[1] * shape[2] > CAPACITY_CELLS
    st = {n: pkg.Storage(np.zeros(shape), H) for n in ("uin", "vin", "mask")}
    st.update({n: pkg.Storage(np.ones(ny + 2 * H), H) for n in ("crlavo", "crlavu", "crlato", "crlatu", "acrlat0")})
    xb = {n: pkg.Storage(np.zeros(shape), H) for n in ("uin", "vin")}
    yb = {n: pkg.Storage(np.zeros(shape), H) for n in ("uout", "vout")}
    sc = {"eddlat": 0.05, "eddlon": 0.05, "tau_smag": 0.025, "weight_smag": 0.01}
    status = _call(pkg, "oeb_hdiffsmag_adj_noalloc_f64", _args(pkg, st, xb, yb, sc, (nx, ny, nz)))
    assert status == OEB_ERR_TOO_LARGE
