"""The chained dycore step (fastwavesuv -> hadvuv5th -> update -> hdiffsmag -> fvtp2d) on the GPU.

* FP64 forward: bit-identical to the same step composed from the oracle's stencils
  (oracle/chain.py), over every written box, with every other cell untouched.
* Tangent-linear and adjoint steps: the dot-product test to 1e-13 (FP64), central
  differences of the GPU forward step, and the adjoint against central differences of the
  oracle's forward step (the reference's stencils differentiated numerically).
* A CUDA graph of forward + adjoint replays to the eager results after the inputs change
  in place, and counts its kernels.
* FP32 step: normwise error against the FP64 oracle step.
"""
from __future__ import annotations

import json
import os
from pathlib import Path

import numpy as np
import pytest

from conftest import assert_bitwise_equal

H = 8
SENTINEL = -7.0e5
OUT_BOX = {"uout": 3, "vout": 3, "fx1": 0, "fy1": 0}  # written box: interior widened by this in i, j
# the measured errors are also written, as JSON, to the file OEB_CHAIN_REPORT names (if set)
REPORT = Path(os.environ["OEB_CHAIN_REPORT"]) if os.environ.get("OEB_CHAIN_REPORT") else None


def _box(arr, e, nx, ny, nz):
    return arr[H:H + nz, H - e:H + ny + e, H - e:H + nx + e]


def _interior(arr, nx, ny, nz):
    return _box(arr, 0, nx, ny, nz)


@pytest.fixture(scope="module")
def chain(pkg):
    import importlib
    return importlib.import_module("oeb_gb300.chain")


@pytest.fixture(scope="module")
def ochain(pkg):
    from oracle import chain as oc
    return oc


class Step:
    def __init__(self, pkg, fields, chain, cuda, nx, ny, nz, seed, modes, dtype=np.float64, workload="physical"):
        import torch
        self.torch, self.pkg, self.chain, self.cuda = torch, pkg, chain, cuda
        self.nx, self.ny, self.nz, self.dtype = nx, ny, nz, dtype
        self.x = fields.make_chain_inputs(nx, ny, nz, seed, workload=workload, halo=H)
        self.s = fields.make_chain_scalars(seed)
        self.shape = self.x["u"].shape
        self.dev_x = {k: self.dev(v) for k, v in self.x.items()}
        self.plan = chain.ChainPlan(self.dev_x["u"], (nx, ny, nz), modes)

    def dev(self, a):
        a = np.ascontiguousarray(a, dtype=self.dtype)
        return self.pkg.Storage(self.torch.from_numpy(a).to(self.cuda), H, nx=self.nx if a.ndim == 3 else None)

    def blank(self, names):
        return {n: self.dev(np.full(self.shape, SENTINEL)) for n in names}

    def forward(self, x=None):
        xs = self.dev_x if x is None else {k: self.dev(v) for k, v in x.items()}
        outs = self.blank(self.chain.OUTPUTS)
        self.plan.forward(xs, self.s, outs)
        self.torch.cuda.synchronize()
        return {k: v.numpy().astype(np.float64) for k, v in outs.items()}

    def tl(self, du, dv):
        dy = self.blank(self.chain.OUTPUTS)
        self.plan.tangent_linear(self.dev_x, self.s, {"u": self.dev(du), "v": self.dev(dv)}, dy)
        self.torch.cuda.synchronize()
        return {k: v.numpy().astype(np.float64) for k, v in dy.items()}

    def adj(self, seeds):
        g = self.blank(("u", "v"))
        self.plan.adjoint(self.dev_x, self.s, {k: self.dev(v) for k, v in seeds.items()}, g)
        self.torch.cuda.synchronize()
        return {k: v.numpy().astype(np.float64) for k, v in g.items()}


def _untouched(arr, e, nx, ny, nz, what):
    mask = np.ones(arr.shape, dtype=bool)
    _box(mask, e, nx, ny, nz)[...] = False
    assert np.all(arr[mask] == SENTINEL), "%s: cells outside the written box were modified" % what


@pytest.mark.gpu
@pytest.mark.parametrize("size", [(128, 128, 80), (40, 36, 5), (1, 1, 1), (70, 97, 9)],
                         ids=["128x128x80", "40x36x5", "1x1x1", "70x97x9"])
def test_chain_forward_bitexact_f64(pkg, fields, chain, ochain, cuda, size):
    nx, ny, nz = size
    st = Step(pkg, fields, chain, cuda, nx, ny, nz, seed=3, modes=chain.FORWARD)
    got = st.forward()
    want = ochain.run_chain(st.x, st.s, nx, ny, nz, H)
    for n, e in OUT_BOX.items():
        assert_bitwise_equal(np.ascontiguousarray(_box(got[n], e, nx, ny, nz)),
                             np.ascontiguousarray(_box(want[n], e, nx, ny, nz)), "chain %s %s" % (n, size))
        _untouched(got[n], e, nx, ny, nz, n)


def _seeds_from(st, dy):
    seeds = {}
    for n in st.chain.OUTPUTS:
        y = np.zeros(st.shape)
        _interior(y, st.nx, st.ny, st.nz)[...] = _interior(dy[n], st.nx, st.ny, st.nz)
        seeds[n] = y
    return seeds


def _dot_test(st, tol):
    rng = np.random.default_rng(17)
    du = rng.normal(0.0, 1.0, size=st.shape)
    dv = rng.normal(0.0, 1.0, size=st.shape)
    dy = st.tl(du, dv)
    seeds = _seeds_from(st, dy)
    g = st.adj(seeds)
    for n in ("u", "v"):
        _untouched(g[n], 7, st.nx, st.ny, st.nz, "grad " + n)
    lhs = sum(float(np.sum(_interior(seeds[n], st.nx, st.ny, st.nz) ** 2)) for n in st.chain.OUTPUTS)
    du32 = np.asarray(du, dtype=st.dtype).astype(np.float64)
    dv32 = np.asarray(dv, dtype=st.dtype).astype(np.float64)
    rhs = float(np.sum(_box(du32, 7, st.nx, st.ny, st.nz) * _box(g["u"], 7, st.nx, st.ny, st.nz)) +
                np.sum(_box(dv32, 7, st.nx, st.ny, st.nz) * _box(g["v"], 7, st.nx, st.ny, st.nz)))
    rel = abs(lhs - rhs) / lhs
    assert rel <= tol, "<J d, J d> = %.17g, <d, J^T J d> = %.17g, rel %.3g" % (lhs, rhs, rel)
    return rel


@pytest.mark.gpu
@pytest.mark.parametrize("size", [(128, 128, 80), (40, 36, 5), (1, 1, 1)], ids=["128x128x80", "40x36x5", "1x1x1"])
def test_chain_dot_product_f64(pkg, fields, chain, cuda, size):
    st = Step(pkg, fields, chain, cuda, *size, seed=3, modes=chain.TL | chain.ADJOINT)
    _dot_test(st, 1e-13)


@pytest.mark.gpu
def test_chain_dot_product_f32(pkg, fields, chain, cuda):
    st = Step(pkg, fields, chain, cuda, 128, 128, 80, seed=3, modes=chain.TL | chain.ADJOINT, dtype=np.float32)
    _dot_test(st, 1e-5)


def _fd_compare(fd, tl, nx, ny, nz, tol=1e-6, flip_fraction=1e-4):
    for n in fd:
        t = _interior(tl[n], nx, ny, nz)
        f = _interior(fd[n], nx, ny, nz)
        scale = max(float(np.max(np.abs(t))), 1e-300)
        bad = np.abs(f - t) > tol * scale
        assert np.count_nonzero(bad) <= int(flip_fraction * t.size) + 2, (
            "%s: TL differs from central differences on %d of %d cells (max rel %.3g)" %
            (n, np.count_nonzero(bad), t.size, float(np.max(np.abs(f - t))) / scale))


@pytest.mark.gpu
def test_chain_tl_vs_central_differences_gpu(pkg, fields, chain, cuda):
    st = Step(pkg, fields, chain, cuda, 128, 128, 80, seed=7, modes=chain.FORWARD | chain.TL)
    rng = np.random.default_rng(7)
    du = rng.normal(0.0, 1.0, size=st.shape) * float(np.std(st.x["u"]))
    dv = rng.normal(0.0, 1.0, size=st.shape) * float(np.std(st.x["v"]))
    eps = 1e-6
    xp = dict(st.x, u=st.x["u"] + eps * du, v=st.x["v"] + eps * dv)
    xm = dict(st.x, u=st.x["u"] - eps * du, v=st.x["v"] - eps * dv)
    fp, fm = st.forward(xp), st.forward(xm)
    fd = {n: (fp[n] - fm[n]) / (2 * eps) for n in chain.OUTPUTS}
    _fd_compare(fd, st.tl(du, dv), st.nx, st.ny, st.nz)


@pytest.mark.gpu
def test_chain_adjoint_vs_central_differences_oracle(pkg, fields, chain, ochain, cuda):
    # <ybar, (F(x + eps d) - F(x - eps d)) / 2 eps> with F the oracle's step, against
    # <d, J^T ybar>, over several random directions d
    nx, ny, nz = 48, 40, 6
    st = Step(pkg, fields, chain, cuda, nx, ny, nz, seed=8, modes=chain.ADJOINT)
    rng = np.random.default_rng(8)
    seeds = {n: np.zeros(st.shape) for n in chain.OUTPUTS}
    for n in chain.OUTPUTS:
        _interior(seeds[n], nx, ny, nz)[...] = rng.normal(0.0, 1.0, size=(nz, ny, nx))
    g = st.adj(seeds)
    eps = 1e-6
    for _ in range(4):
        du = rng.normal(0.0, 1.0, size=st.shape) * float(np.std(st.x["u"]))
        dv = rng.normal(0.0, 1.0, size=st.shape) * float(np.std(st.x["v"]))
        fp = ochain.run_chain(dict(st.x, u=st.x["u"] + eps * du, v=st.x["v"] + eps * dv), st.s, nx, ny, nz, H)
        fm = ochain.run_chain(dict(st.x, u=st.x["u"] - eps * du, v=st.x["v"] - eps * dv), st.s, nx, ny, nz, H)
        fd = sum(float(np.sum(_interior(seeds[n], nx, ny, nz) *
                              (_interior(fp[n], nx, ny, nz) - _interior(fm[n], nx, ny, nz)) / (2 * eps)))
                 for n in chain.OUTPUTS)
        ad = float(np.sum(_box(du, 7, nx, ny, nz) * _box(g["u"], 7, nx, ny, nz)) +
                   np.sum(_box(dv, 7, nx, ny, nz) * _box(g["v"], 7, nx, ny, nz)))
        assert abs(fd - ad) <= 1e-6 * max(abs(fd), abs(ad)), "FD %.12g vs adjoint %.12g" % (fd, ad)


@pytest.mark.gpu
def test_chain_graph_replays_forward_and_adjoint(pkg, fields, chain, cuda):
    import torch
    nx, ny, nz = 40, 36, 5
    st = Step(pkg, fields, chain, cuda, nx, ny, nz, seed=11, modes=chain.FORWARD | chain.ADJOINT)
    stream = torch.cuda.Stream()
    outs = st.blank(chain.OUTPUTS)
    rng = np.random.default_rng(11)
    seeds = {}
    for n in chain.OUTPUTS:
        y = np.zeros(st.shape)
        _interior(y, nx, ny, nz)[...] = rng.normal(0.0, 1.0, size=(nz, ny, nx))
        seeds[n] = st.dev(y)
    grads = st.blank(("u", "v"))
    torch.cuda.synchronize()
    # one eager run on the stream first: one-time set-up happens outside the capture
    st.plan.forward(st.dev_x, st.s, outs, stream=stream)
    st.plan.adjoint(st.dev_x, st.s, seeds, grads, stream=stream)
    stream.synchronize()
    g = chain.Graph(stream)
    with g:
        st.plan.forward(st.dev_x, st.s, outs, stream=stream)
        st.plan.adjoint(st.dev_x, st.s, seeds, grads, stream=stream)
    assert g.kernels > 0
    # new input values in place; the graph reads the same buffers
    x2 = fields.make_chain_inputs(nx, ny, nz, 12, halo=H)
    for k in ("u", "v", "ppuv", "mask"):
        st.dev_x[k].data.copy_(torch.from_numpy(x2[k]).to(cuda))
    torch.cuda.synchronize()
    lib = pkg.load_library()
    before = lib.oeb_launch_count()
    g.launch(stream)
    stream.synchronize()
    assert lib.oeb_launch_count() - before == g.kernels
    want_o = st.blank(chain.OUTPUTS)
    want_g = st.blank(("u", "v"))
    st.plan.forward(st.dev_x, st.s, want_o)
    st.plan.adjoint(st.dev_x, st.s, seeds, want_g)
    torch.cuda.synchronize()
    for n in chain.OUTPUTS:
        assert_bitwise_equal(outs[n].numpy(), want_o[n].numpy(), "graph " + n)
    for n in ("u", "v"):
        assert_bitwise_equal(grads[n].numpy(), want_g[n].numpy(), "graph grad " + n)
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", [("physical", 128, 128, 80, 3), ("fronts", 70, 97, 9, 5)])
def test_chain_f32_error_vs_f64_oracle(pkg, fields, chain, ochain, cuda, case):
    workload, nx, ny, nz, seed = case
    st = Step(pkg, fields, chain, cuda, nx, ny, nz, seed=seed, modes=chain.FORWARD, dtype=np.float32,
              workload=workload)
    got = st.forward()
    want = ochain.run_chain(st.x, st.s, nx, ny, nz, H)
    # the FP64 step on the FP32-rounded inputs: the error of the FP32 arithmetic alone
    xq = {k: v.astype(np.float32).astype(np.float64) for k, v in st.x.items()}
    sq = {k: float(np.float32(v)) for k, v in st.s.items()}
    want_q = ochain.run_chain(xq, sq, nx, ny, nz, H)
    res = {}
    for n, e in OUT_BOX.items():
        g = _box(got[n], e, nx, ny, nz)
        w = _box(want[n], e, nx, ny, nz)
        wq = _box(want_q[n], e, nx, ny, nz)
        scale = float(np.max(np.abs(w)))
        tot = np.abs(g - w) / scale
        ar = np.abs(g - wq) / scale
        res[n] = {"total_max": float(tot.max()), "total_rms": float(np.sqrt(np.mean(tot ** 2))),
                  "arith_max": float(ar.max()), "arith_rms": float(np.sqrt(np.mean(ar ** 2))),
                  "arith_over_1e-5": int((ar > 1e-5).sum()), "points": int(ar.size)}
    if REPORT is not None:
        REPORT.parent.mkdir(parents=True, exist_ok=True)
        old = json.loads(REPORT.read_text()) if REPORT.exists() else {}
        old["%s_%dx%dx%d" % (workload, nx, ny, nz)] = res
        REPORT.write_text(json.dumps(old, indent=1, sort_keys=True))
    for n, r in res.items():
        # a limiter branch of fvtp2d may flip where FP32 cannot resolve the deciding difference
        assert r["arith_over_1e-5"] <= 1e-4 * r["points"] + 2, (n, r)
        assert r["arith_rms"] <= 1e-6, (n, r)


def test_chain_plan_rejects_a_halo_below_8(pkg):
    import ctypes
    lib = pkg.load_library()
    like = pkg.Storage(np.zeros((11, 14, 14)), 3)  # halo 3: the widest stage needs 8
    plan = ctypes.c_void_p()
    fn = lib.oeb_chain_plan_create_f64
    fn.restype = ctypes.c_int
    st = fn(ctypes.byref(like.memref()), ctypes.byref(pkg.Domain(8, 8, 5)), ctypes.c_int(1), ctypes.byref(plan))
    assert st == 4  # OEB_ERR_HALO
    assert not plan.value


@pytest.mark.gpu
def test_chain_workspace_fields_per_mode(pkg, fields, chain, cuda):
    """The adjoint step's fields share the buffers of forward fields that are dead while they
    are live: 10 workspace fields for the forward step, 12 for the adjoint (with or without
    the forward), 19 for the tangent-linear, 23 for all three."""
    field_bytes = None
    for modes, n in ((chain.FORWARD, 10), (chain.ADJOINT, 12), (chain.FORWARD | chain.ADJOINT, 12), (chain.TL, 19),
                     (chain.FORWARD | chain.TL | chain.ADJOINT, 23)):
        st = Step(pkg, fields, chain, cuda, 24, 20, 4, 3, modes)
        field_bytes = st.x["u"].size * 8
        assert st.plan.nbytes == n * field_bytes, (modes, st.plan.nbytes / field_bytes)
        st.plan.close()


@pytest.mark.gpu
def test_chain_calls_alternate_on_one_plan(pkg, fields, chain, cuda):
    """Forward, adjoint and tangent-linear calls on one plan, in turn, give the bits each
    gives on a plan of its own: no call reads what another left in a shared buffer."""
    nx, ny, nz = 40, 36, 5
    both = Step(pkg, fields, chain, cuda, nx, ny, nz, 3, chain.FORWARD | chain.TL | chain.ADJOINT)
    rng = np.random.default_rng(5)
    seeds = {k: rng.normal(size=both.shape) for k in chain.OUTPUTS}
    du, dv = rng.normal(size=both.shape), rng.normal(size=both.shape)
    alone = {m: Step(pkg, fields, chain, cuda, nx, ny, nz, 3, m) for m in (chain.FORWARD, chain.TL, chain.ADJOINT)}
    want_f = alone[chain.FORWARD].forward()
    want_a = alone[chain.ADJOINT].adj(seeds)
    want_t = alone[chain.TL].tl(du, dv)
    for _ in range(2):
        for got, want in ((both.adj(seeds), want_a), (both.forward(), want_f), (both.tl(du, dv), want_t)):
            for k in want:
                np.testing.assert_array_equal(got[k].view(np.uint64), want[k].view(np.uint64), err_msg=k)
