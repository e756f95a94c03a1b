"""Seeded synthetic inputs for the stencils.

The reference fills its inputs analytically (``fillMath``, include/util.h:150-188) over the
i/j halo but leaves the k-halo planes unset (util.h:159), although fastwavesuv, nh_p_grad
and p_grad_c read k-1 or k+1 there.  Every generator here fills every cell of the
allocation, halo included on all three axes, deterministically from a seed.

Workloads (sizes are interior extents; the halo is 3 cells on every side):

* ``smooth``   -- 64x64x60-style field for laplace/hdiffsa: a sum of three random-phase
                  sin(2 pi kx i/N) cos(2 pi ky j/N) modes (kx, ky in 1..4) plus U[0, 1e-3)
                  noise; crlato/crlatu = 1 + 0.1 U[0,1); mask = U[0, 0.025).
* ``physical`` -- all ten kernels: velocities 10 x smooth modes + N(0, 0.1); pressure-like
                  and geopotential-like fields monotone in k (1000 -> 100 hPa) with a 1 %
                  smooth perturbation, so the thickness denominators stay away from 0;
                  fvtp2d Courant numbers and mass fluxes scaled to |c| <= 0.8 with a
                  zero-mean tracer q so the PPM limiter fires; scalars U[0.01, 0.1).
* ``fronts``   -- ``physical`` plus steep tanh fronts (width 2 cells) on every dynamic
                  field, so limiters and upwind switches change branch often.
"""
from __future__ import annotations

from typing import Dict, Optional

import numpy as np

from .specs import KERNELS, DRIVER_SCALARS

HALO = 3


class Grid:
    """Index arrays over the whole allocation: i, j, k run over [-h, n+h)."""

    def __init__(self, nx, ny, nz, halo):
        self.nx, self.ny, self.nz, self.h = nx, ny, nz, halo
        self.i = np.arange(-halo, nx + halo, dtype=np.float64)[None, None, :]
        self.j = np.arange(-halo, ny + halo, dtype=np.float64)[None, :, None]
        self.k = np.arange(-halo, nz + halo, dtype=np.float64)[:, None, None]
        self.shape = (nz + 2 * halo, ny + 2 * halo, nx + 2 * halo)

    def jline(self):
        return np.arange(-self.h, self.ny + self.h, dtype=np.float64)


def smooth_modes(g: Grid, rng: np.random.Generator, nmodes=3, kmax=4, vertical=True) -> np.ndarray:
    """Sum of random-phase sin(kx i) cos(ky j) modes with a smooth vertical modulation."""
    out = np.zeros(g.shape)
    for _ in range(nmodes):
        kx, ky = rng.integers(1, kmax + 1, size=2)
        phi, psi, chi = rng.uniform(0, 2 * np.pi, size=3)
        mode = np.sin(2 * np.pi * kx * g.i / g.nx + phi) * np.cos(2 * np.pi * ky * g.j / g.ny + psi)
        if vertical:
            kz = rng.integers(1, 3)
            mode = mode * (1.0 + 0.5 * np.sin(2 * np.pi * kz * g.k / max(g.nz, 1) + chi))
        out += mode
    return out


def tanh_front(g: Grid, rng: np.random.Generator, width=2.0) -> np.ndarray:
    """A straight tanh front of the given width (cells) in a random direction and position."""
    theta = rng.uniform(0, 2 * np.pi)
    c = np.array([rng.uniform(0.25, 0.75) * g.nx, rng.uniform(0.25, 0.75) * g.ny])
    dist = (g.i - c[0]) * np.cos(theta) + (g.j - c[1]) * np.sin(theta)
    return np.broadcast_to(np.tanh(dist / width), g.shape).copy()


def pressure_profile(g: Grid, rng, top=100.0, bottom=1000.0, pert=0.01) -> np.ndarray:
    """Monotone in k from `bottom` (k=0) to `top` (k=nz-1), continued into the k-halo, with a
    `pert` relative smooth perturbation."""
    frac = g.k / max(g.nz - 1, 1)
    base = bottom + (top - bottom) * frac
    return base * (1.0 + pert * smooth_modes(g, rng, vertical=False) / 3.0)


def _velocity(g, rng, fronts):
    v = 10.0 * smooth_modes(g, rng) + rng.normal(0.0, 0.1, size=g.shape)
    if fronts:
        v += 10.0 * tanh_front(g, rng)
    return v


def _tracer(g, rng, fronts):
    q = smooth_modes(g, rng) + rng.normal(0.0, 0.05, size=g.shape)
    q -= q.mean()
    if fronts:
        q += tanh_front(g, rng)
    return q


def _courant(g, rng, fronts):
    c = smooth_modes(g, rng) + rng.normal(0.0, 0.05, size=g.shape)
    if fronts:
        c += tanh_front(g, rng)
    return 0.8 * c / np.max(np.abs(c))


def _metric(g, rng):
    return 1.0 + 0.1 * rng.uniform(0.0, 1.0, size=g.jline().shape)


# Field classes per kernel input (physical/fronts workloads).
_CLASSES = {
    "laplace": {"in": "vel"},
    "hdiffsa": {"in": "vel", "mask": "mask", "crlato": "metric", "crlatu": "metric"},
    "hdiffsmag": {"uin": "vel", "vin": "vel", "mask": "unit", "crlavo": "metric", "crlavu": "metric",
                  "crlato": "metric", "crlatu": "metric", "acrlat0": "metric"},
    "hadvuv": {"uin": "vel", "vin": "vel", "acrlat0": "metric", "acrlat1": "metric", "tgrlatda0": "metric",
               "tgrlatda1": "metric"},
    "fastwavesuv": {"uin": "vel", "vin": "vel", "utens": "tend", "vtens": "tend", "wgtfac": "weight",
                    "ppuv": "ppert", "hhl": "height", "rho": "density", "fx": "metric"},
    "uvbke": {"uc": "vel", "vc": "vel", "cosa": "cosa", "rsina": "rsina"},
    "nh_p_grad": {"uin": "vel", "vin": "vel", "rdx": "rdx", "rdy": "rdx", "gz": "geopot", "pp": "pres",
                  "pk3": "pres", "wk1": "thick"},
    "p_grad_c": {"uin": "vel", "vin": "vel", "rdxc": "rdx", "rdyc": "rdx", "delpc": "thick", "gz": "geopot",
                 "pkc": "pres"},
    "fvtp2d": {"q": "tracer", "crx": "courant", "cry": "courant", "ra_x": "area", "ra_y": "area", "xfx": "courant",
               "yfx": "courant", "area": "area"},
}
_CLASSES["hadvuv5th"] = _CLASSES["hadvuv"]


def _make(cls: str, g: Grid, rng, fronts: bool, rank: int) -> np.ndarray:
    if rank == 1:
        return _metric(g, rng)
    if cls == "vel":
        return _velocity(g, rng, fronts)
    if cls == "tend":
        return 1e-3 * _velocity(g, rng, fronts)
    if cls == "mask":
        return rng.uniform(0.0, 0.025, size=g.shape)
    if cls == "unit":
        return rng.uniform(0.0, 1.0, size=g.shape)
    if cls == "weight":
        return rng.uniform(0.4, 0.6, size=g.shape)
    if cls == "ppert":
        return 100.0 * smooth_modes(g, rng) + rng.normal(0.0, 1.0, size=g.shape)
    if cls == "height":  # half-level heights decreasing with k, like COSMO's hhl
        frac = g.k / max(g.nz, 1)
        return 20000.0 * (1.0 - frac) * (1.0 + 0.01 * smooth_modes(g, rng, vertical=False) / 3.0)
    if cls == "density":
        return 1.2 * (1.0 + 0.01 * smooth_modes(g, rng))
    if cls == "cosa":
        return 0.2 * smooth_modes(g, rng) / 3.0
    if cls == "rsina":
        return 1.0 + 0.05 * smooth_modes(g, rng) / 3.0
    if cls == "rdx":
        return 1.0 + 0.1 * rng.uniform(0.0, 1.0, size=g.shape)
    if cls == "geopot":  # g z with z rising from 1 km to 16 km over the column
        return 9.81 * pressure_profile(g, rng, top=16000.0, bottom=1000.0)
    if cls == "pres":
        return pressure_profile(g, rng)
    if cls == "thick":
        return 10.0 * (1.0 + 0.01 * smooth_modes(g, rng))
    if cls == "tracer":
        return _tracer(g, rng, fronts)
    if cls == "courant":
        return _courant(g, rng, fronts)
    if cls == "area":
        return 1.0 + 0.1 * smooth_modes(g, rng) / 3.0
    raise KeyError(cls)


def smooth_config1(g: Grid, rng) -> np.ndarray:
    """Sum of 3 random-phase sin cos modes + U[0, 1e-3) noise (the 64x64x60 workload)."""
    return smooth_modes(g, rng, vertical=True) + rng.uniform(0.0, 1e-3, size=g.shape)


def make_inputs(kernel: str, nx: int, ny: int, nz: int, seed: int, workload: str = "physical",
                halo: int = HALO, dtype=np.float64) -> Dict[str, np.ndarray]:
    """Input buffers (whole allocations, halo included) of `kernel`, keyed by argument name."""
    spec = KERNELS[kernel]
    g = Grid(nx, ny, nz, halo)
    # one independent stream per (kernel, field) so a field does not depend on the others
    out = {}
    for idx, a in enumerate(spec.args):
        if a.role not in ("in3", "in1"):
            continue
        rng = np.random.default_rng([seed, sum(map(ord, kernel)), idx])
        rank = 3 if a.role == "in3" else 1
        if workload == "smooth":
            if rank == 1:
                arr = _metric(g, rng)
            elif a.name == "mask":
                arr = rng.uniform(0.0, 0.025, size=g.shape)
            else:
                arr = smooth_config1(g, rng)
        else:
            arr = _make(_CLASSES[kernel][a.name], g, rng, workload == "fronts", rank)
        out[a.name] = np.ascontiguousarray(arr, dtype=dtype)
    return out


def make_scalars(kernel: str, seed: int, workload: str = "physical") -> Dict[str, float]:
    """Scalars: the reference drivers' values for ``driver``, else U[0.01, 0.1) (p1/p2 keep the
    driver macros)."""
    spec = KERNELS[kernel]
    if workload == "driver":
        return dict(DRIVER_SCALARS.get(kernel, {}))
    rng = np.random.default_rng([seed, sum(map(ord, kernel)), 999])
    vals = {}
    for s in spec.scalars:
        vals[s.name] = float(rng.uniform(0.01, 0.1))
    if kernel == "fvtp2d":
        vals.update(DRIVER_SCALARS["fvtp2d"])
    return vals


SENTINEL = -7.0e5  # fill of every output before a call: cells outside the written box keep it


def make_outputs(kernel: str, nx: int, ny: int, nz: int, halo: int = HALO, dtype=np.float64,
                 include_scratch: bool = False) -> Dict[str, np.ndarray]:
    spec = KERNELS[kernel]
    shape = (nz + 2 * halo, ny + 2 * halo, nx + 2 * halo)
    out = {}
    for a in spec.args:
        if a.role == "out3" or (include_scratch and a.role == "scratch3"):
            out[a.name] = np.full(shape, SENTINEL, dtype=dtype)
    return out


def points(nx, ny, nz) -> int:
    return nx * ny * nz


# Inputs of the chained step (chain.py), from the generators of the stencils that read them:
# (u, v) and the fastwavesuv fields from fastwavesuv, the metric terms of the advection from
# hadvuv5th, mask and the diffusion metrics from hdiffsmag, the fluxes' geometry from fvtp2d.
CHAIN_SOURCES = {
    "u": ("fastwavesuv", "uin"), "v": ("fastwavesuv", "vin"), "utens": ("fastwavesuv", "utens"),
    "vtens": ("fastwavesuv", "vtens"), "wgtfac": ("fastwavesuv", "wgtfac"), "ppuv": ("fastwavesuv", "ppuv"),
    "hhl": ("fastwavesuv", "hhl"), "rho": ("fastwavesuv", "rho"), "fx": ("fastwavesuv", "fx"),
    "acrlat0": ("hadvuv5th", "acrlat0"), "acrlat1": ("hadvuv5th", "acrlat1"),
    "tgrlatda0": ("hadvuv5th", "tgrlatda0"), "tgrlatda1": ("hadvuv5th", "tgrlatda1"),
    "mask": ("hdiffsmag", "mask"), "crlavo": ("hdiffsmag", "crlavo"), "crlavu": ("hdiffsmag", "crlavu"),
    "crlato": ("hdiffsmag", "crlato"), "crlatu": ("hdiffsmag", "crlatu"), "smag_acrlat0": ("hdiffsmag", "acrlat0"),
    "crx": ("fvtp2d", "crx"), "cry": ("fvtp2d", "cry"), "ra_x": ("fvtp2d", "ra_x"), "ra_y": ("fvtp2d", "ra_y"),
    "xfx": ("fvtp2d", "xfx"), "yfx": ("fvtp2d", "yfx"), "area": ("fvtp2d", "area"),
}
CHAIN_HALO = 8
CHAIN_DT_ADV = 0.01  # stage 3: the advective tendencies move u by a few per cent


def make_chain_inputs(nx: int, ny: int, nz: int, seed: int, workload: str = "physical", halo: int = CHAIN_HALO,
                      dtype=np.float64) -> Dict[str, np.ndarray]:
    per_kernel = {k: make_inputs(k, nx, ny, nz, seed, workload, halo=halo, dtype=dtype)
                  for k in {src for src, _ in CHAIN_SOURCES.values()}}
    return {name: per_kernel[k][arg] for name, (k, arg) in CHAIN_SOURCES.items()}


def make_chain_scalars(seed: int) -> Dict[str, float]:
    fw = make_scalars("fastwavesuv", seed)
    adv = make_scalars("hadvuv5th", seed)
    smag = make_scalars("hdiffsmag", seed)
    fv = make_scalars("fvtp2d", seed)
    return {"edadlat": fw["edadlat"], "dt": fw["dt"], "eddlat": adv["eddlat"], "eddlon": adv["eddlon"],
            "dt_adv": CHAIN_DT_ADV, "tau_smag": smag["tau_smag"], "weight_smag": smag["weight_smag"],
            "ppm_p1": fv["p1"], "ppm_p2": fv["p2"]}


# ---- the same generators on the device (torch), for workloads too large for numpy -------
# Same formulas and distributions as above; the random streams are torch's, so values differ
# from the numpy generators for the same seed.
def _t_grid(nx, ny, nz, halo, device, torch):
    i = torch.arange(-halo, nx + halo, dtype=torch.float64, device=device)[None, None, :]
    j = torch.arange(-halo, ny + halo, dtype=torch.float64, device=device)[None, :, None]
    k = torch.arange(-halo, nz + halo, dtype=torch.float64, device=device)[:, None, None]
    return i, j, k


def _t_modes(g, nx, ny, nz, gen, torch, vertical=True, nmodes=3, kmax=4):
    i, j, k = g
    shape = (k.shape[0], j.shape[1], i.shape[2])
    out = torch.zeros(shape, dtype=torch.float64, device=i.device)
    for _ in range(nmodes):
        kx, ky = (int(v) for v in torch.randint(1, kmax + 1, (2,), generator=gen))
        phi, psi, chi = (float(v) * 2 * np.pi for v in torch.rand(3, generator=gen, dtype=torch.float64))
        mode = torch.sin(2 * np.pi * kx * i / nx + phi) * torch.cos(2 * np.pi * ky * j / ny + psi)
        if vertical:
            kz = int(torch.randint(1, 3, (1,), generator=gen))
            mode = mode * (1.0 + 0.5 * torch.sin(2 * np.pi * kz * k / max(nz, 1) + chi))
        out += mode.expand(shape)
    return out


def make_chain_inputs_device(nx: int, ny: int, nz: int, seed: int, device, dtype=np.float64,
                             halo: int = CHAIN_HALO):
    """Inputs of the chained step (CHAIN_SOURCES) made on `device` with the "physical"
    generators; returns torch tensors, whole allocations with the halo."""
    import torch
    g = _t_grid(nx, ny, nz, halo, device, torch)
    i, j, k = g
    shape = (k.shape[0], j.shape[1], i.shape[2])
    tdt = torch.float64 if np.dtype(dtype) == np.float64 else torch.float32
    out = {}
    for idx, (name, (kernel, arg)) in enumerate(CHAIN_SOURCES.items()):
        gen = torch.Generator(device="cpu").manual_seed(int(seed) * 1000003 + idx * 7919)
        dgen = torch.Generator(device=device).manual_seed(int(seed) * 1000003 + idx * 7919 + 1)
        cls = _CLASSES[kernel][arg]
        rank1 = name in ("fx", "acrlat0", "acrlat1", "tgrlatda0", "tgrlatda1", "crlavo", "crlavu", "crlato", "crlatu",
                         "smag_acrlat0")
        if rank1:
            a = 1.0 + 0.1 * torch.rand(ny + 2 * halo, generator=dgen, device=device, dtype=torch.float64)
        elif cls == "vel":
            a = 10.0 * _t_modes(g, nx, ny, nz, gen, torch) + 0.1 * torch.randn(shape, generator=dgen, device=device,
                                                                                dtype=torch.float64)
        elif cls == "tend":
            a = 1e-3 * (10.0 * _t_modes(g, nx, ny, nz, gen, torch) +
                        0.1 * torch.randn(shape, generator=dgen, device=device, dtype=torch.float64))
        elif cls == "unit":
            a = torch.rand(shape, generator=dgen, device=device, dtype=torch.float64)
        elif cls == "weight":
            a = 0.4 + 0.2 * torch.rand(shape, generator=dgen, device=device, dtype=torch.float64)
        elif cls == "ppert":
            a = 100.0 * _t_modes(g, nx, ny, nz, gen, torch) + torch.randn(shape, generator=dgen, device=device,
                                                                          dtype=torch.float64)
        elif cls == "height":
            frac = k / max(nz, 1)
            a = 20000.0 * (1.0 - frac) * (1.0 + 0.01 * _t_modes(g, nx, ny, nz, gen, torch, vertical=False) / 3.0)
        elif cls == "density":
            a = 1.2 * (1.0 + 0.01 * _t_modes(g, nx, ny, nz, gen, torch))
        elif cls == "tracer":
            a = _t_modes(g, nx, ny, nz, gen, torch) + 0.05 * torch.randn(shape, generator=dgen, device=device,
                                                                         dtype=torch.float64)
            a -= a.mean()
        elif cls == "courant":
            a = _t_modes(g, nx, ny, nz, gen, torch) + 0.05 * torch.randn(shape, generator=dgen, device=device,
                                                                         dtype=torch.float64)
            a = 0.8 * a / a.abs().max()
        elif cls == "area":
            a = 1.0 + 0.1 * _t_modes(g, nx, ny, nz, gen, torch) / 3.0
        else:
            raise KeyError(cls)
        out[name] = a.expand(shape).to(tdt).contiguous() if a.dim() == 3 else a.to(tdt).contiguous()
    return out


def ensemble_members(count: int = 48, seed: int = 4):
    """The uneven ensemble: nx, ny uniform in {48, 64, ..., 320}, nz in {40, 60, 80, 137},
    FP64 or FP32 with equal odds.  Returns [(nx, ny, nz, itemsize)]."""
    rng = np.random.default_rng(seed)
    sizes = np.arange(48, 321, 16)
    out = []
    for _ in range(count):
        nx, ny = (int(v) for v in rng.choice(sizes, size=2))
        nz = int(rng.choice([40, 60, 80, 137]))
        out.append((nx, ny, nz, 8 if rng.random() < 0.5 else 4))
    return out
