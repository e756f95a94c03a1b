"""Memory safety of every kernel without a sanitizer: poisoned halos and guard bands.

compute-sanitizer is not available, so two checks stand in for it:

* every input cell outside the reach the C ABI declares for that input is NaN (halo planes
  in k included); a kernel that used such a cell would produce NaN or different bits, so
  each output must be bit-identical to the same call on fully defined inputs;
* every field lives inside a larger buffer whose guard bands, before and after the
  field's span, are a NaN pattern; after the call the guard bands must be unchanged, and
  output cells outside the written box keep their sentinel.

Covered: the ten forward stencils (FP64 and FP32) and the tangent-linear and adjoint
entry points of hdiffsmag, hadvuv, hadvuv5th, fastwavesuv and fvtp2d.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = 4
G = 1024  # guard elements on each side of every field
SENTINEL = -7.0e5
NX, NY, NZ = 37, 45, 5
KERNELS = ("laplace", "hdiffsa", "hdiffsmag", "hadvuv", "hadvuv5th", "fastwavesuv", "uvbke", "nh_p_grad",
           "p_grad_c", "fvtp2d")
ADJ = ("hdiffsmag", "hadvuv", "hadvuv5th", "fastwavesuv", "fvtp2d", "laplace", "hdiffsa", "uvbke", "nh_p_grad",
       "p_grad_c")


class Guarded:
    """A field inside a buffer with NaN guard bands."""

    def __init__(self, pkg, arr, cuda):
        import torch
        self.torch = torch
        dt = torch.float64 if arr.dtype == np.float64 else torch.float32
        self.buf = torch.full((arr.size + 2 * G,), float("nan"), dtype=dt, device=cuda)
        self.view = self.buf[G:G + arr.size].view(arr.shape)
        self.view.copy_(torch.from_numpy(np.ascontiguousarray(arr)).to(cuda))
        self.st = pkg.Storage(self.view, H, nx=NX if arr.ndim == 3 else None)
        self.guard0 = self.buf[:G].clone()
        self.guard1 = self.buf[-G:].clone()

    def guards_intact(self):
        t = self.torch
        itype = t.int64 if self.buf.dtype == t.float64 else t.int32
        return bool(t.equal(self.buf[:G].view(itype), self.guard0.view(itype)) and
                    t.equal(self.buf[-G:].view(itype), self.guard1.view(itype)))


def _poison(arr, reach):
    """NaN outside the reach box [-ilo, n+ihi) x [-jlo, n+jhi) x [-klo, nz+khi)."""
    out = np.full_like(arr, np.nan)
    ilo, ihi, jlo, jhi, klo, khi = reach
    if arr.ndim == 1:
        out[H - jlo:H + NY + jhi] = arr[H - jlo:H + NY + jhi]
        return out
    box = (slice(H - klo, H + NZ + khi), slice(H - jlo, H + NY + jhi), slice(H - ilo, H + NX + ihi))
    out[box] = arr[box]
    return out


def _bits(a):
    return a.view(np.int64 if a.dtype == np.float64 else np.int32)


def _box(arr, reach):
    ilo, ihi, jlo, jhi, klo, khi = reach
    return arr[H - klo:H + NZ + khi, H - jlo:H + NY + jhi, H - ilo:H + NX + ihi]


def _inputs(pkg, fields, name, dtype, seed):
    x = fields.make_inputs(name, NX, NY, NZ, seed=seed, workload="fronts", halo=H, dtype=dtype)
    return x, fields.make_scalars(name, seed=seed)


def _outputs(spec, dtype):
    shape = (NZ + 2 * H, NY + 2 * H, NX + 2 * H)
    return {a.name: np.full(shape, SENTINEL, dtype=dtype) for a in spec.by_role("out3")}


def _check_outputs(spec, got, want, where):
    for a in spec.by_role("out3"):
        g, w = got[a.name], want[a.name]
        assert np.array_equal(_bits(g), _bits(w)), "%s: %s differs when unread cells are NaN" % (where, a.name)
        assert np.all(np.isfinite(_box(g, a.reach))), "%s: %s has NaN in its written box" % (where, a.name)
        mask = np.ones(g.shape, dtype=bool)
        _box(mask, a.reach)[...] = False
        assert np.all(g[mask] == SENTINEL), "%s: %s written outside its box" % (where, a.name)


@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("name", KERNELS)
def test_forward_reads_only_its_reach_and_writes_only_its_box(pkg, fields, cuda, name, dtype):
    import torch
    spec = pkg.KERNELS[name]
    x, sc = _inputs(pkg, fields, name, dtype, seed=31)
    runs = {}
    for label, poison in (("clean", False), ("poisoned", True)):
        ins = {a.name: Guarded(pkg, _poison(x[a.name], a.reach) if poison else x[a.name], cuda)
               for a in spec.args if a.role in ("in3", "in1")}
        outs = {n: Guarded(pkg, v, cuda) for n, v in _outputs(spec, dtype).items()}
        pkg.call(name, {**{k: v.st for k, v in ins.items()}, **{k: v.st for k, v in outs.items()}}, sc,
                 domain=(NX, NY, NZ))
        torch.cuda.synchronize()
        for k, v in list(ins.items()) + list(outs.items()):
            assert v.guards_intact(), "%s %s: guard band of %s overwritten" % (name, label, k)
        runs[label] = {k: v.view.cpu().numpy() for k, v in outs.items()}
    _check_outputs(spec, runs["poisoned"], runs["clean"], "%s %s" % (name, np.dtype(dtype).name))


@pytest.mark.parametrize("name", ADJ)
def test_tangent_linear_and_adjoint_read_only_their_reach(pkg, fields, cuda, name):
    import torch
    spec = pkg.KERNELS[name]
    x, sc = _inputs(pkg, fields, name, np.float64, seed=32)
    rng = np.random.default_rng(32)
    dx = {n: rng.normal(0.0, 1.0, size=x[n].shape) for n in pkg.ACTIVE[name]}
    yb = {n: rng.normal(0.0, 1.0, size=(NZ + 2 * H, NY + 2 * H, NX + 2 * H)) for n in spec.semantic_outputs}
    reach = {a.name: a.reach for a in spec.args}
    interior = (0, 0, 0, 0, 0, 0)
    results = {}
    for label, poison in (("clean", False), ("poisoned", True)):
        p = (lambda a, r: _poison(a, r)) if poison else (lambda a, r: a)
        st = {a.name: Guarded(pkg, p(x[a.name], a.reach), cuda) for a in spec.args if a.role in ("in3", "in1")}
        d = {n: Guarded(pkg, p(v, reach[n]), cuda) for n, v in dx.items()}
        dy = {a.name: Guarded(pkg, np.full((NZ + 2 * H, NY + 2 * H, NX + 2 * H), SENTINEL), cuda)
              for a in spec.by_role("out3")}
        y = {n: Guarded(pkg, p(v, interior), cuda) for n, v in yb.items()}
        xb = {n: Guarded(pkg, np.full((NZ + 2 * H, NY + 2 * H, NX + 2 * H), SENTINEL), cuda) for n in dx}
        s = {k: v.st for k, v in st.items()}
        pkg.tangent_linear(name, s, {k: v.st for k, v in d.items()}, {k: v.st for k, v in dy.items()}, sc,
                           domain=(NX, NY, NZ))
        pkg.adjoint(name, s, {k: v.st for k, v in y.items()}, {k: v.st for k, v in xb.items()}, sc,
                    domain=(NX, NY, NZ))
        torch.cuda.synchronize()
        for group in (st, d, dy, y, xb):
            for k, v in group.items():
                assert v.guards_intact(), "%s %s: guard band of %s overwritten" % (name, label, k)
        results[label] = ({k: v.view.cpu().numpy() for k, v in dy.items()},
                          {k: v.view.cpu().numpy() for k, v in xb.items()})
    (dy0, xb0), (dy1, xb1) = results["clean"], results["poisoned"]
    for a in spec.by_role("out3"):
        assert np.array_equal(_bits(dy1[a.name]), _bits(dy0[a.name])), "%s TL: d%s" % (name, a.name)
    for n in dx:
        assert np.array_equal(_bits(xb1[n]), _bits(xb0[n])), "%s adjoint: %sb" % (name, n)
        assert np.all(np.isfinite(_box(xb1[n], reach[n]))), "%s adjoint: NaN in %sb" % (name, n)
