"""Tangent-linear and adjoint stencils on the GPU.

For every one of the ten stencils the library exports ``oeb_<k>_tl_<p>`` (dy = J(x) dx,
branches frozen at x) and ``oeb_<k>_adj_<p>`` (xbar = J(x)^T ybar, a gather with no
atomics).  Checked here:

* the dot-product test <J dx, J dx> = <dx, J^T (J dx)> over the written boxes, to 1e-13
  relative in FP64 and 1e-5 in FP32;
* the tangent-linear image against central differences of the GPU forward stencil and
  of the oracle's forward stencil (the C restatement of the reference kernel, bit-exact
  with it), allowing only the few cells whose branch flips inside the difference step;
* single adjoint columns J^T e_p against the TL image, and dy = 0 for dx = 0;
* nothing outside the written boxes is touched.
"""
from __future__ import annotations

import numpy as np
import pytest

import branch_flips

pytestmark = pytest.mark.gpu

H = 3
ADJ = ("hdiffsmag", "hadvuv", "hadvuv5th", "fastwavesuv", "fvtp2d", "laplace", "hdiffsa", "uvbke", "nh_p_grad",
       "p_grad_c")
SENTINEL = -7.0e5


def _box(arr, reach, nx, ny, nz, halo=H):
    ilo, ihi, jlo, jhi, klo, khi = reach
    return arr[halo - klo:halo + nz + khi, halo - jlo:halo + ny + jhi, halo - ilo:halo + nx + ihi]


def _outside_untouched(arr, reach, nx, ny, nz, what):
    mask = np.ones(arr.shape, dtype=bool)
    _box(mask, reach, nx, ny, nz)[...] = False
    bad = np.count_nonzero(arr[mask] != SENTINEL)
    assert bad == 0, "%s: %d cells outside the written box were modified" % (what, bad)


class Case:
    """One state x of a stencil, its perturbations and device buffers."""

    def __init__(self, pkg, fields, cuda, name, nx, ny, nz, seed, workload="physical", dtype=np.float64):
        import torch
        self.pkg, self.cuda, self.name = pkg, cuda, name
        self.nx, self.ny, self.nz, self.dtype = nx, ny, nz, dtype
        self.spec = pkg.KERNELS[name]
        self.active = pkg.ACTIVE[name]
        self.x = fields.make_inputs(name, nx, ny, nz, seed=seed, workload=workload, halo=H)
        self.scalars = fields.make_scalars(name, seed=seed)
        rng = np.random.default_rng([seed, 77])
        # perturbations scaled to each active field's spread, so eps is a relative step
        self.dx = {n: rng.normal(0.0, 1.0, size=self.x[n].shape) * float(np.std(self.x[n])) for n in self.active}
        self.reach = {a.name: a.reach for a in self.spec.args}
        self.torch = torch

    def dev(self, arr):
        arr = np.ascontiguousarray(arr, dtype=self.dtype)
        return self.pkg.Storage(self.torch.from_numpy(arr).to(self.cuda), H, nx=self.nx if arr.ndim == 3 else None)

    def shape3(self):
        return (self.nz + 2 * H, self.ny + 2 * H, self.nx + 2 * H)

    def state(self, x=None):
        x = self.x if x is None else x
        return {k: self.dev(v) for k, v in x.items()}

    def forward(self, x):
        """GPU forward stencil at x; returns the outputs as float64 arrays."""
        st = self.state(x)
        outs = {a.name: self.dev(np.full(self.shape3(), SENTINEL)) for a in self.spec.by_role("out3")}
        self.pkg.call(self.name, {**st, **outs}, self.scalars, domain=(self.nx, self.ny, self.nz))
        self.torch.cuda.synchronize()
        return {k: v.numpy().astype(np.float64) for k, v in outs.items()}

    def tl(self, dx=None):
        dx = self.dx if dx is None else dx
        dy = {a.name: self.dev(np.full(self.shape3(), SENTINEL)) for a in self.spec.by_role("out3")}
        self.pkg.tangent_linear(self.name, self.state(), {n: self.dev(v) for n, v in dx.items()}, dy,
                                self.scalars, domain=(self.nx, self.ny, self.nz))
        self.torch.cuda.synchronize()
        return {k: v.numpy().astype(np.float64) for k, v in dy.items()}

    def adj(self, ybar):
        xb = {n: self.dev(np.full(self.shape3(), SENTINEL)) for n in self.active}
        self.pkg.adjoint(self.name, self.state(), {n: self.dev(v) for n, v in ybar.items()}, xb, self.scalars,
                         domain=(self.nx, self.ny, self.nz))
        self.torch.cuda.synchronize()
        return {k: v.numpy().astype(np.float64) for k, v in xb.items()}

    def sem_box(self, name, arr):
        return _box(arr, self.reach[name], self.nx, self.ny, self.nz)


def _dot_test(case: Case, tol: float):
    dy = case.tl()
    for a in case.spec.by_role("out3"):
        _outside_untouched(dy[a.name], a.reach, case.nx, case.ny, case.nz, "%s TL d%s" % (case.name, a.name))
    # ybar = J dx on the semantic outputs' boxes, 0 elsewhere
    ybar = {}
    for n in case.spec.semantic_outputs:
        y = np.zeros(case.shape3())
        case.sem_box(n, y)[...] = case.sem_box(n, dy[n])
        ybar[n] = y
    xbar = case.adj(ybar)
    lhs = sum(float(np.sum(case.sem_box(n, ybar[n]) ** 2)) for n in case.spec.semantic_outputs)
    rhs = 0.0
    for n in case.active:
        _outside_untouched(xbar[n], case.reach[n], case.nx, case.ny, case.nz, "%s ADJ %sb" % (case.name, n))
        xd = np.ascontiguousarray(case.dx[n], dtype=case.dtype).astype(np.float64)
        rhs += float(np.sum(case.sem_box(n, xd) * case.sem_box(n, xbar[n])))
    assert lhs > 0.0, "%s: J dx vanished" % case.name
    rel = abs(lhs - rhs) / lhs
    assert rel <= tol, "%s: <J dx, J dx> = %.17g, <dx, J^T J dx> = %.17g, rel %.3g > %.1g" % (
        case.name, lhs, rhs, rel, tol)
    return rel


@pytest.mark.parametrize("name", ADJ)
@pytest.mark.parametrize("size", [(40, 36, 5), (128, 128, 80)], ids=["40x36x5", "128x128x80"])
def test_dot_product_f64(pkg, fields, cuda, name, size):
    _dot_test(Case(pkg, fields, cuda, name, *size, seed=3), 1e-13)


@pytest.mark.parametrize("name", ADJ)
def test_dot_product_f64_fronts_ragged(pkg, fields, cuda, name):
    # steep fronts flip limiters and upwind switches often; ragged tiles on every edge
    _dot_test(Case(pkg, fields, cuda, name, 70, 97, 9, seed=5, workload="fronts"), 1e-13)


@pytest.mark.parametrize("name", ADJ)
def test_dot_product_f64_tiny(pkg, fields, cuda, name):
    _dot_test(Case(pkg, fields, cuda, name, 1, 1, 1, seed=4), 1e-13)


@pytest.mark.parametrize("name", ADJ)
def test_dot_product_f32(pkg, fields, cuda, name):
    _dot_test(Case(pkg, fields, cuda, name, 128, 128, 80, seed=3, dtype=np.float32), 1e-5)


@pytest.mark.parametrize("name", ADJ)
@pytest.mark.parametrize("size", [(70, 97, 9), (1, 1, 1)], ids=["70x97x9", "1x1x1"])
def test_dot_product_f32_edges(pkg, fields, cuda, name, size):
    # ragged tiles on every edge and a single cell, in FP32 (whose adjoints may take other
    # launch forms than FP64's)
    _dot_test(Case(pkg, fields, cuda, name, *size, seed=5, dtype=np.float32, workload="fronts"), 1e-5)


def _flip_cells(case: Case, xp: dict, xm: dict):
    """hdiffsa: the output cells whose limiter flags differ between the two ends of the step
    (tests/branch_flips.py); None for the other stencils, whose flips are counted."""
    if case.name != "hdiffsa":
        return None
    ks = slice(H, H + case.nz)
    fp = branch_flips.hdiffsa_flags(xp["in"][ks], case.x["crlato"], case.x["crlatu"], case.nx, case.ny, H)
    fm = branch_flips.hdiffsa_flags(xm["in"][ks], case.x["crlato"], case.x["crlatu"], case.nx, case.ny, H)
    return branch_flips.hdiffsa_affected(fp, fm, case.nx, case.ny)


def _compare_fd(case: Case, fd: dict, dy: dict, tol=1e-6, max_flip_fraction=1e-4, flips=None):
    """|FD - TL| <= tol * max|TL| on every cell of every output box, except cells where a
    branch flips within the step: those in `flips` where they are known (hdiffsa's
    discontinuous limiter), else at most max_flip_fraction of the box, plus 2."""
    for a in case.spec.by_role("out3"):
        t = case.sem_box(a.name, dy[a.name])
        f = case.sem_box(a.name, fd[a.name])
        scale = max(float(np.max(np.abs(t))), 1e-300)
        bad = np.abs(f - t) > tol * scale
        if flips is not None:
            outside = int(np.count_nonzero(bad & ~flips))
            assert outside == 0, "%s.%s: TL differs from central differences on %d cells where no branch flips" % (
                case.name, a.name, outside)
            continue
        allowed = int(max_flip_fraction * t.size) + 2
        assert np.count_nonzero(bad) <= allowed, (
            "%s.%s: TL differs from central differences on %d of %d cells (max rel %.3g)" %
            (case.name, a.name, np.count_nonzero(bad), t.size, float(np.max(np.abs(f - t))) / scale))


@pytest.mark.parametrize("name", ADJ)
def test_tl_vs_central_differences_gpu(pkg, fields, cuda, name):
    case = Case(pkg, fields, cuda, name, 128, 128, 80, seed=7)
    eps = 1e-6
    xp = {k: (v + eps * case.dx[k] if k in case.dx else v) for k, v in case.x.items()}
    xm = {k: (v - eps * case.dx[k] if k in case.dx else v) for k, v in case.x.items()}
    fp, fm = case.forward(xp), case.forward(xm)
    fd = {k: (fp[k] - fm[k]) / (2 * eps) for k in fp}
    _compare_fd(case, fd, case.tl(), flips=_flip_cells(case, xp, xm))


@pytest.mark.parametrize("name", ADJ)
def test_tl_vs_central_differences_oracle(pkg, fields, orc, cuda, name):
    # the difference quotient of the CPU restatement of the reference forward stencil
    case = Case(pkg, fields, cuda, name, 48, 40, 6, seed=8)
    eps = 1e-6

    def oracle_forward(x):
        bufs = {k: v.copy() for k, v in x.items()}
        bufs.update(fields.make_outputs(name, case.nx, case.ny, case.nz, halo=H))
        orc.run_oracle(case.spec, bufs, case.scalars, case.nx, case.ny, case.nz, H)
        return {a.name: bufs[a.name] for a in case.spec.by_role("out3")}

    xp = {k: (v + eps * case.dx[k] if k in case.dx else v) for k, v in case.x.items()}
    xm = {k: (v - eps * case.dx[k] if k in case.dx else v) for k, v in case.x.items()}
    fp, fm = oracle_forward(xp), oracle_forward(xm)
    fd = {k: (fp[k] - fm[k]) / (2 * eps) for k in fp}
    _compare_fd(case, fd, case.tl(), flips=_flip_cells(case, xp, xm))


@pytest.mark.parametrize("name", ADJ)
def test_adjoint_columns_match_tl(pkg, fields, cuda, name):
    # J^T e_p on a few output cells p equals row p of J: <J e_q, e_p> = <e_q, J^T e_p>, read
    # off the TL image of a random dx: sum_q (J^T e_p)[q] dx[q] = (J dx)[p]
    case = Case(pkg, fields, cuda, name, 24, 20, 3, seed=9)
    dy = case.tl()
    rng = np.random.default_rng(11)
    out = case.spec.semantic_outputs[0]
    for _ in range(4):
        k, j, i = (int(rng.integers(0, n)) for n in (case.nz, case.ny, case.nx))
        e = {n: np.zeros(case.shape3()) for n in case.spec.semantic_outputs}
        e[out][H + k, H + j, H + i] = 1.0
        xb = case.adj(e)
        got = sum(float(np.sum(case.sem_box(n, xb[n]) * case.sem_box(n, case.dx[n]))) for n in case.active)
        want = dy[out][H + k, H + j, H + i]
        assert abs(got - want) <= 1e-12 * max(abs(want), float(np.max(np.abs(case.sem_box(out, dy[out]))))), (
            "%s: (J^T e_p . dx) = %.17g, (J dx)_p = %.17g at %s" % (name, got, want, (i, j, k)))


@pytest.mark.parametrize("name", ADJ)
def test_tl_zero_perturbation(pkg, fields, cuda, name):
    # the dual-number run with dx = 0 gives dy = 0 exactly on every written cell
    case = Case(pkg, fields, cuda, name, 40, 36, 5, seed=12)
    dy = case.tl({n: np.zeros(case.shape3()) for n in case.active})
    for a in case.spec.by_role("out3"):
        assert not np.any(case.sem_box(a.name, dy[a.name])), "%s.%s: dy != 0 for dx = 0" % (name, a.name)
