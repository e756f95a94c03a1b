"""Finite-difference checks of every adjoint on 64 random directions (benchmark configuration 4).

For each of the ten stencils, in FP64 and FP32, at 128x128x80 + 3-cell halo (state: the
'physical' generators at seed 3), and for the chained step (i/j halo 8, seed 3):

* one random output seed ybar ~ N(0, 1) on the semantic outputs' boxes, and its adjoint
  g = J^T ybar, computed once;
* 64 random directions d, each active input ~ N(0, std of that input);
* for every direction, central differences with step 1e-6 of the FP64 forward -- the GPU
  stencil, and the oracle (the C restatement of the reference's kernel, bit-exact with it) --
  compared with
  - the tangent-linear image J d, cell by cell: |FD - TL| <= tol * max|TL| on every written
    cell except those where a limiter, upwind or PPM branch flips inside the step (at most
    1e-4 of the cells + 2 per output field), and
  - the adjoint, through the scalar <ybar, FD> against <g, d> (at a flip cell the TL value
    stands in for the difference quotient).

hdiffsa's limiter is discontinuous (a flux is zeroed when flux * (in(i+1) - in(i)) > 0, so the
output jumps where the difference of `in` changes sign), and about 3e-4 of its cells jump
inside the step: for it the test finds those cells exactly (tests/branch_flips.py) and
requires every deviating cell to be one of them.

FP32: the state is the FP64 state rounded to FP32 and the directions are rounded to FP32; the
differences are those of the FP64 forward at that state, so they measure the FP32
tangent-linear and adjoint against the exact derivative of the same function.

Tolerances: per cell 1e-6 (FP64) and 2e-5 (FP32) of max|TL|; the adjoint scalar to 1e-6
relative (FP64) and to 1e-5 of |ybar| |FD| (FP32, whose sums of 1.3 M products of FP32
values carry that much rounding).  The worst deviations and the flip counts of every
direction are written, as JSON, to the file OEB_FD_REPORT names (if set).
"""
from __future__ import annotations

import json
import os
from pathlib import Path

import numpy as np
import pytest

import branch_flips

pytestmark = pytest.mark.gpu

H = 3
NX, NY, NZ = 128, 128, 80
SEED = 3
DIRECTIONS = 64
EPS = 1e-6
SENTINEL = -7.0e5
FLIP_FRACTION = 1e-4
TOL = {np.float64: {"cell": 1e-6, "scalar": 1e-6}, np.float32: {"cell": 2e-5, "scalar": 1e-5}}
ADJ = ("laplace", "hdiffsa", "hdiffsmag", "hadvuv", "hadvuv5th", "fastwavesuv", "uvbke", "nh_p_grad", "p_grad_c",
       "fvtp2d")
REPORT = Path(os.environ["OEB_FD_REPORT"]) if os.environ.get("OEB_FD_REPORT") else None
_report = {}


def _write_report():
    if REPORT is not None:
        REPORT.write_text(json.dumps(_report, indent=1, sort_keys=True))


def _box(a, reach, nx=NX, ny=NY, nz=NZ, h=H):
    ilo, ihi, jlo, jhi, klo, khi = reach
    return a[h - klo:h + nz + khi, h - jlo:h + ny + jhi, h - ilo:h + nx + ihi]


def _compare(fd, tl, tol, allowed=None):
    """(cells where |FD - TL| > tol max|TL|, how many of them lie outside `allowed` -- the
    cells where a branch is known to flip inside the step, if given --, the worst
    |FD - TL| / max|TL| over the other cells, FD with TL at those cells), for torch or numpy
    float64 arrays of one output box."""
    if isinstance(fd, np.ndarray):
        diff = np.abs(fd - tl)
        scale = max(float(np.max(np.abs(tl))), 1e-300)
        bad = diff > tol * scale
        worst = float(np.max(np.where(bad, 0.0, diff))) / scale
        out = int(np.count_nonzero(bad & ~allowed)) if allowed is not None else 0
        return int(np.count_nonzero(bad)), out, worst, np.where(bad, tl, fd)
    diff = (fd - tl).abs()
    scale = max(float(tl.abs().max()), 1e-300)
    bad = diff > tol * scale
    worst = float(diff.masked_fill(bad, 0.0).max()) / scale
    out = 0
    if allowed is not None:
        import torch
        out = int((bad & ~torch.from_numpy(allowed).to(bad.device)).sum())
    return int(bad.sum()), out, worst, fd.masked_fill(bad, 0.0) + tl * bad


def _check_flips(what, nbad, outside, size, allowed):
    """With the flip cells known (allowed), every deviating cell must be one of them; else at
    most FLIP_FRACTION of the cells (+ 2) may deviate."""
    if allowed is not None:
        assert outside == 0, "%s: TL differs from the differences on %d cells where no branch flips" % (
            what, outside)
    else:
        assert nbad <= int(FLIP_FRACTION * size) + 2, "%s: TL differs from the differences on %d cells" % (
            what, nbad)


class Stencil:
    """One stencil's state on the device (FP64 for the differences, the tested precision for
    the tangent-linear and adjoint) and its oracle forward."""

    def __init__(self, pkg, fields, orc, cuda, name, dtype):
        import torch
        self.torch, self.pkg, self.fields, self.orc, self.cuda = torch, pkg, fields, orc, cuda
        self.name, self.dtype = name, dtype
        self.spec = pkg.KERNELS[name]
        self.active = pkg.ACTIVE[name]
        self.reach = {a.name: a.reach for a in self.spec.args}
        x = fields.make_inputs(name, NX, NY, NZ, seed=SEED, halo=H)
        # the state the differences are taken at: for FP32 the FP32 values, held in FP64
        self.x = {k: np.asarray(v, dtype=dtype).astype(np.float64) for k, v in x.items()}
        sc = fields.make_scalars(name, seed=SEED)
        dbl = {x.name for x in self.spec.scalars if x.always_double}
        # FP32: the scalars the FP32 entry points see, for the FP64 differences as well
        self.scalars = {k: (v if dtype == np.float64 or k in dbl else float(np.float32(v))) for k, v in sc.items()}
        self.shape3 = (NZ + 2 * H, NY + 2 * H, NX + 2 * H)
        self.x64 = {k: self.dev(v, np.float64) for k, v in self.x.items()}
        self.xp = {k: self.dev(v, dtype) for k, v in self.x.items()}
        self.outs = [a.name for a in self.spec.by_role("out3")]

    def dev(self, a, dtype):
        t = self.torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to(self.cuda)
        return self.pkg.Storage(t, H, nx=NX if t.ndim == 3 else None)

    def blank(self, names, dtype):
        return {n: self.dev(np.full(self.shape3, SENTINEL), dtype) for n in names}

    def gpu_fd(self, d64):
        """FP64 GPU forward differences along d (device tensors keyed by active input)."""
        res = []
        for sign in (1.0, -1.0):
            st = dict(self.x64)
            for n, dn in d64.items():
                st[n] = self.pkg.Storage(self.x64[n].data + (sign * EPS) * dn, H, nx=NX)
            outs = self.blank(self.outs, np.float64)
            self.pkg.call(self.name, {**st, **outs}, self.scalars, domain=(NX, NY, NZ))
            res.append(outs)
        return {n: (_box(res[0][n].data, self.reach[n]) - _box(res[1][n].data, self.reach[n])) / (2 * EPS)
                for n in self.outs}

    def oracle_fd(self, d):
        """The oracle's forward differences along d (numpy arrays keyed by active input)."""
        res = []
        for sign in (1.0, -1.0):
            bufs = {k: v.copy() for k, v in self.x.items()}
            for n, dn in d.items():
                bufs[n] += (sign * EPS) * dn
            bufs.update(self.fields.make_outputs(self.name, NX, NY, NZ, halo=H))
            self.orc.run_oracle(self.spec, bufs, self.scalars, NX, NY, NZ, H)
            res.append(bufs)
        return {n: (_box(res[0][n], self.reach[n]) - _box(res[1][n], self.reach[n])) / (2 * EPS) for n in self.outs}

    def flip_cells(self, d):
        """Per output, the cells where a branch flips inside the step (None where the test
        counts them instead): hdiffsa's limiter flags at x - eps d and x + eps d, and for FP32
        also the FP32 flags at the state against the FP64 ones."""
        if self.name != "hdiffsa":
            return {n: None for n in self.outs}
        ks = slice(H, H + NZ)
        lo, lu = self.x["crlato"], self.x["crlatu"]
        xp = (self.x["in"] + EPS * d["in"])[ks]
        xm = (self.x["in"] + (-EPS) * d["in"])[ks]
        fp = branch_flips.hdiffsa_flags(xp, lo, lu, NX, NY, H)
        fm = branch_flips.hdiffsa_flags(xm, lo, lu, NX, NY, H)
        mask = branch_flips.hdiffsa_affected(fp, fm, NX, NY)
        if self.dtype == np.float32:
            f32 = branch_flips.hdiffsa_flags(self.x["in"][ks].astype(np.float32), lo, lu, NX, NY, H, exact_sign=True)
            f64 = branch_flips.hdiffsa_flags(self.x["in"][ks], lo, lu, NX, NY, H)
            mask |= branch_flips.hdiffsa_affected(f32, f64, NX, NY)
        return {"out": mask}

    def tl(self, d):
        dy = self.blank(self.outs, self.dtype)
        self.pkg.tangent_linear(self.name, self.xp, {n: self.dev(v, self.dtype) for n, v in d.items()}, dy,
                                self.scalars, domain=(NX, NY, NZ))
        return {n: _box(dy[n].data, self.reach[n]).double() for n in self.outs}

    def adj(self, ybar):
        xb = self.blank(self.active, self.dtype)
        self.pkg.adjoint(self.name, self.xp, {n: self.dev(v, self.dtype) for n, v in ybar.items()}, xb, self.scalars,
                         domain=(NX, NY, NZ))
        return {n: _box(xb[n].data, self.reach[n]).double() for n in self.active}


def _directions(x, active, m, dtype):
    rng = np.random.default_rng([SEED, 4242, m])
    d = {n: rng.normal(0.0, 1.0, size=x[n].shape) * float(np.std(x[n])) for n in active}
    return {n: v.astype(dtype).astype(np.float64) for n, v in d.items()}


@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("name", ADJ)
def test_adjoint_against_central_differences_64_directions(pkg, fields, orc, cuda, name, dtype):
    import torch
    tol = TOL[dtype]
    s = Stencil(pkg, fields, orc, cuda, name, dtype)
    rng = np.random.default_rng([SEED, 77])
    ybar = {}
    for n in s.spec.semantic_outputs:
        y = np.zeros(s.shape3)
        _box(y, s.reach[n])[...] = rng.normal(0.0, 1.0, size=_box(y, s.reach[n]).shape)
        ybar[n] = np.asarray(y, dtype=dtype).astype(np.float64)
    yb_dev = {n: _box(torch.from_numpy(v).to(cuda), s.reach[n]) for n, v in ybar.items()}
    yb_host = {n: _box(v, s.reach[n]) for n, v in ybar.items()}
    g = s.adj(ybar)
    rows = []
    for m in range(DIRECTIONS):
        d = _directions(s.x, s.active, m, dtype)
        d_dev = {n: torch.from_numpy(v).to(cuda) for n, v in d.items()}
        tl = s.tl(d)
        fd_gpu = s.gpu_fd(d_dev)
        fd_orc = s.oracle_fd(d)
        tl_host = {n: t.cpu().numpy() for n, t in tl.items()}
        flips = s.flip_cells(d)
        row = {"flips_gpu": 0, "flips_oracle": 0, "cell_gpu": 0.0, "cell_oracle": 0.0}
        s_gpu = s_orc = 0.0
        fd_norm = 0.0
        for n in s.outs:
            what = "%s %s dir %d %s" % (name, np.dtype(dtype).name, m, n)
            nf, outside, worst, masked = _compare(fd_gpu[n], tl[n], tol["cell"], flips[n])
            row["flips_gpu"] = max(row["flips_gpu"], nf)
            row["cell_gpu"] = max(row["cell_gpu"], worst)
            _check_flips(what + " (GPU forward)", nf, outside, tl[n].numel(), flips[n])
            if n in yb_dev:
                s_gpu += float((yb_dev[n] * masked).sum())
                fd_norm += float((masked * masked).sum())
            nf, outside, worst, masked = _compare(fd_orc[n], tl_host[n], tol["cell"], flips[n])
            row["flips_oracle"] = max(row["flips_oracle"], nf)
            row["cell_oracle"] = max(row["cell_oracle"], worst)
            _check_flips(what + " (oracle forward)", nf, outside, tl_host[n].size, flips[n])
            if n in yb_host:
                s_orc += float(np.sum(yb_host[n] * masked))
        s_adj = sum(float((_box(d_dev[n], s.reach[n]) * g[n]).sum()) for n in s.active)
        y_norm = float(np.sqrt(sum(float(np.sum(v * v)) for v in yb_host.values())))
        if dtype == np.float64:
            row["scalar_gpu"] = abs(s_gpu - s_adj) / max(abs(s_gpu), abs(s_adj), 1e-300)
            row["scalar_oracle"] = abs(s_orc - s_adj) / max(abs(s_orc), abs(s_adj), 1e-300)
        else:
            den = max(y_norm * np.sqrt(fd_norm), 1e-300)
            row["scalar_gpu"] = abs(s_gpu - s_adj) / den
            row["scalar_oracle"] = abs(s_orc - s_adj) / den
        rows.append(row)
        for key in ("scalar_gpu", "scalar_oracle"):
            assert row[key] <= tol["scalar"], "%s %s dir %d: <ybar, FD> vs <J^T ybar, d>: %s %.3g > %.1g" % (
                name, np.dtype(dtype).name, m, key, row[key], tol["scalar"])
    _report["%s/%s" % (name, np.dtype(dtype).name)] = {
        "directions": len(rows), "tol": tol,
        "worst_cell_gpu": max(r["cell_gpu"] for r in rows), "worst_cell_oracle": max(r["cell_oracle"] for r in rows),
        "worst_scalar_gpu": max(r["scalar_gpu"] for r in rows),
        "worst_scalar_oracle": max(r["scalar_oracle"] for r in rows),
        "max_flips_gpu": max(r["flips_gpu"] for r in rows), "max_flips_oracle": max(r["flips_oracle"] for r in rows),
        "flips_gpu_per_direction": [r["flips_gpu"] for r in rows]}
    _write_report()


# ---- the chained step ------------------------------------------------------------------
CH = 8
CHAIN_BOX = {"uout": 3, "vout": 3, "fx1": 0, "fy1": 0}  # written box: interior widened in i, j


def _cbox(a, e):
    return a[CH:CH + NZ, CH - e:CH + NY + e, CH - e:CH + NX + e]


@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_chain_adjoint_against_central_differences_64_directions(pkg, fields, cuda, dtype):
    import importlib

    import torch
    from oracle import chain as ochain
    chain = importlib.import_module("oeb_gb300.chain")
    tol = TOL[dtype]
    x = fields.make_chain_inputs(NX, NY, NZ, SEED, halo=CH)
    x = {k: np.asarray(v, dtype=dtype).astype(np.float64) for k, v in x.items()}
    sc = {k: float(np.asarray(v, dtype=dtype)) for k, v in fields.make_chain_scalars(SEED).items()}
    shape = x["u"].shape

    def dev(a, dt):
        t = torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(cuda)
        return pkg.Storage(t, CH, nx=NX if t.ndim == 3 else None)

    def blank(names, dt):
        return {n: dev(np.full(shape, SENTINEL), dt) for n in names}

    x64 = {k: dev(v, np.float64) for k, v in x.items()}
    xp = {k: dev(v, dtype) for k, v in x.items()}
    fwd = chain.ChainPlan(x64["u"], (NX, NY, NZ), chain.FORWARD)
    plan = chain.ChainPlan(xp["u"], (NX, NY, NZ), chain.TL | chain.ADJOINT)
    rng = np.random.default_rng([SEED, 78])
    seeds = {n: np.zeros(shape) for n in chain.OUTPUTS}
    for n in chain.OUTPUTS:
        _cbox(seeds[n], 0)[...] = rng.normal(0.0, 1.0, size=(NZ, NY, NX))
        seeds[n] = seeds[n].astype(dtype).astype(np.float64)
    g = blank(("u", "v"), dtype)
    plan.adjoint(xp, sc, {n: dev(v, dtype) for n, v in seeds.items()}, g)
    g = {n: _cbox(g[n].data, 7).double() for n in ("u", "v")}
    y_dev = {n: _cbox(torch.from_numpy(v).to(cuda), CHAIN_BOX[n]) for n, v in seeds.items()}
    y_host = {n: _cbox(v, CHAIN_BOX[n]) for n, v in seeds.items()}
    y_norm = float(np.sqrt(sum(float(np.sum(v * v)) for v in y_host.values())))
    rows = []
    for m in range(DIRECTIONS):
        rd = np.random.default_rng([SEED, 4343, m])
        d = {n: (rd.normal(0.0, 1.0, size=shape) * float(np.std(x[n]))).astype(dtype).astype(np.float64)
             for n in ("u", "v")}
        d_dev = {n: torch.from_numpy(v).to(cuda) for n, v in d.items()}
        dy = blank(chain.OUTPUTS, dtype)
        plan.tangent_linear(xp, sc, {n: dev(v, dtype) for n, v in d.items()}, dy)
        tl = {n: _cbox(dy[n].data, CHAIN_BOX[n]).double() for n in chain.OUTPUTS}
        res = []
        for sign in (1.0, -1.0):
            st = dict(x64, u=pkg.Storage(x64["u"].data + (sign * EPS) * d_dev["u"], CH, nx=NX),
                      v=pkg.Storage(x64["v"].data + (sign * EPS) * d_dev["v"], CH, nx=NX))
            outs = blank(chain.OUTPUTS, np.float64)
            fwd.forward(st, sc, outs)
            res.append(outs)
        fd_gpu = {n: (_cbox(res[0][n].data, CHAIN_BOX[n]) - _cbox(res[1][n].data, CHAIN_BOX[n])) / (2 * EPS)
                  for n in chain.OUTPUTS}
        op = ochain.run_chain(dict(x, u=x["u"] + EPS * d["u"], v=x["v"] + EPS * d["v"]), sc, NX, NY, NZ, CH)
        om = ochain.run_chain(dict(x, u=x["u"] - EPS * d["u"], v=x["v"] - EPS * d["v"]), sc, NX, NY, NZ, CH)
        fd_orc = {n: (_cbox(op[n], CHAIN_BOX[n]) - _cbox(om[n], CHAIN_BOX[n])) / (2 * EPS) for n in chain.OUTPUTS}
        row = {"flips_gpu": 0, "flips_oracle": 0, "cell_gpu": 0.0, "cell_oracle": 0.0}
        s_gpu = s_orc = fd_norm = 0.0
        for n in chain.OUTPUTS:
            nf, _, worst, masked = _compare(fd_gpu[n], tl[n], tol["cell"])
            assert nf <= int(FLIP_FRACTION * tl[n].numel()) + 2, "chain dir %d: %s: %d flip cells" % (m, n, nf)
            row["flips_gpu"], row["cell_gpu"] = max(row["flips_gpu"], nf), max(row["cell_gpu"], worst)
            s_gpu += float((y_dev[n] * masked).sum())
            fd_norm += float((masked * masked).sum())
            th = tl[n].cpu().numpy()
            nf, _, worst, masked = _compare(fd_orc[n], th, tol["cell"])
            assert nf <= int(FLIP_FRACTION * th.size) + 2, "chain dir %d: %s: %d flip cells (oracle)" % (m, n, nf)
            row["flips_oracle"], row["cell_oracle"] = max(row["flips_oracle"], nf), max(row["cell_oracle"], worst)
            s_orc += float(np.sum(y_host[n] * masked))
        s_adj = sum(float((_cbox(d_dev[n], 7) * g[n]).sum()) for n in ("u", "v"))
        if dtype == np.float64:
            row["scalar_gpu"] = abs(s_gpu - s_adj) / max(abs(s_gpu), abs(s_adj), 1e-300)
            row["scalar_oracle"] = abs(s_orc - s_adj) / max(abs(s_orc), abs(s_adj), 1e-300)
        else:
            den = max(y_norm * np.sqrt(fd_norm), 1e-300)
            row["scalar_gpu"], row["scalar_oracle"] = abs(s_gpu - s_adj) / den, abs(s_orc - s_adj) / den
        rows.append(row)
        for key in ("scalar_gpu", "scalar_oracle"):
            assert row[key] <= tol["scalar"], "chain %s dir %d: %s %.3g" % (np.dtype(dtype).name, m, key, row[key])
    _report["chain/%s" % np.dtype(dtype).name] = {
        "directions": len(rows), "tol": tol,
        "worst_cell_gpu": max(r["cell_gpu"] for r in rows), "worst_cell_oracle": max(r["cell_oracle"] for r in rows),
        "worst_scalar_gpu": max(r["scalar_gpu"] for r in rows),
        "worst_scalar_oracle": max(r["scalar_oracle"] for r in rows),
        "max_flips_gpu": max(r["flips_gpu"] for r in rows), "max_flips_oracle": max(r["flips_oracle"] for r in rows),
        "flips_gpu_per_direction": [r["flips_gpu"] for r in rows]}
    _write_report()
