"""Cells of a stencil's output whose frozen branch changes inside a finite-difference step.

A central difference (F(x + eps d) - F(x - eps d)) / 2 eps matches the tangent-linear image
J(x) d only where the function is smooth on the segment [x - eps d, x + eps d].  hdiffsa's
flux limiter (kernels/hdiffsa.h:106-113) zeroes a flux when flux * (in(i+1) - in(i)) > 0: where
the difference of `in` changes sign with the flux nonzero, the output jumps, and the
difference quotient there is of order jump / eps.  This module finds those cells exactly --
the limiter flags recomputed (in numpy, in the kernel's order of operations) at both ends of
the step -- so that a test can require every cell where the difference quotient departs from
J d to be one of them, instead of allowing some number of unexplained cells.
"""
from __future__ import annotations

import numpy as np


def hdiffsa_flags(a, crlato, crlatu, nx, ny, h, exact_sign=False):
    """Limiter flags of hdiffsa at the state `a` (whole buffer [k, j, i], halo h): (fx, fy),
    True where the flux is zeroed; fx over i in [-1, nx), j in [0, ny); fy over i in [0, nx),
    j in [-1, ny).  exact_sign: the sign of the exact product (the FP32 kernels' test), else
    the rounded product compared with 0 (the FP64 test)."""
    t = a.dtype.type
    lo = crlato[h - 1:h + ny + 1][None, :, None].astype(a.dtype)
    lu = crlatu[h - 1:h + ny + 1][None, :, None].astype(a.dtype)

    def sl(di, dj):  # a at (i + di, j + dj) for i, j in [-1, N+1)
        return a[:, h - 1 + dj:h + ny + 1 + dj, h - 1 + di:h + nx + 1 + di]

    c = sl(0, 0)
    lap = (((sl(-1, 0) + sl(1, 0)) - t(2.0) * c) + lo * (sl(0, 1) - c)) + lu * (sl(0, -1) - c)
    # lap index [k, j+1, i+1]; flx at i in [-1, nx), j in [0, ny)
    flx = lap[:, 1:ny + 1, 1:nx + 2] - lap[:, 1:ny + 1, 0:nx + 1]
    dxin = a[:, h:h + ny, h:h + nx + 1] - a[:, h:h + ny, h - 1:h + nx]
    fly = lo[:, 0:ny + 1, :] * (lap[:, 1:ny + 2, 1:nx + 1] - lap[:, 0:ny + 1, 1:nx + 1])
    dyin = a[:, h:h + ny + 1, h:h + nx] - a[:, h - 1:h + ny, h:h + nx]

    def test(f, g):
        if exact_sign:
            return ((f > 0) & (g > 0)) | ((f < 0) & (g < 0))
        return (f * g) > 0

    return test(flx, dxin), test(fly, dyin)


def hdiffsa_affected(flags_a, flags_b, nx, ny):
    """Output cells [k, j, i] over the interior whose fluxes flx(i-1), flx(i), fly(j-1), fly(j)
    differ in flag between two flag sets."""
    fx = flags_a[0] != flags_b[0]  # [k, j, i+1] for i in [-1, nx)
    fy = flags_a[1] != flags_b[1]  # [k, j+1, i] for j in [-1, ny)
    return fx[:, :, 0:nx] | fx[:, :, 1:nx + 1] | fy[:, 0:ny, :] | fy[:, 1:ny + 1, :]
