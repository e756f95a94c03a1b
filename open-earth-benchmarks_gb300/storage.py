"""Fields in the reference's strided layout (include/util.h:24-31, :99-141).

A :class:`Storage` wraps one buffer -- a numpy array (host) or a torch tensor (host or
CUDA) -- holding the whole allocation of a field, halo included, and describes it with the
reference's descriptor: element (i, j, k) of a rank-3 field lives at
``aligned[offset + strides[2]*i + strides[1]*j + strides[0]*k]`` with ``strides[2] == 1``;
the interior starts at (0, 0, 0) and the halo spans ``[-halo, n + halo)`` on every axis.

Rank-3 buffers have shape ``(nz + 2h, ny + 2h, pitch)`` with ``pitch >= nx + 2h``; a pitch
larger than ``nx + 2h`` pads rows (legal: kernels honour the strides).  Rank-1 buffers
(per-latitude arrays indexed by j) have shape ``(n + 2h,)``.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import numpy as np

try:  # torch is plumbing for device buffers; host-only use needs numpy alone
    import torch
except Exception:  # pragma: no cover - torch is present in every supported environment
    torch = None


class Memref3d(ctypes.Structure):
    """oeb_memref3d_{f64,f32} (include/oeb_gb300.h): the Storage<T,3> layout."""
    _fields_ = [("allocated", ctypes.c_void_p), ("aligned", ctypes.c_void_p), ("offset", ctypes.c_int64),
                ("sizes", ctypes.c_int64 * 3), ("strides", ctypes.c_int64 * 3)]


class Memref1d(ctypes.Structure):
    """oeb_memref1d_{f64,f32}: the Storage<T,1> layout."""
    _fields_ = [("allocated", ctypes.c_void_p), ("aligned", ctypes.c_void_p), ("offset", ctypes.c_int64),
                ("sizes", ctypes.c_int64 * 1), ("strides", ctypes.c_int64 * 1)]


class Domain(ctypes.Structure):
    """oeb_domain: interior extents (domain_size, domain_size, domain_height in the reference)."""
    _fields_ = [("nx", ctypes.c_int64), ("ny", ctypes.c_int64), ("nz", ctypes.c_int64)]


def _is_torch(x) -> bool:
    return torch is not None and isinstance(x, torch.Tensor)


class Storage:
    """One field: a buffer plus the reference descriptor of it."""

    def __init__(self, data, halo: int, nx: Optional[int] = None):
        if _is_torch(data):
            if not data.is_contiguous():
                raise ValueError("Storage buffers must be contiguous")
            dtype = {torch.float64: np.float64, torch.float32: np.float32}.get(data.dtype)
        else:
            data = np.ascontiguousarray(data)
            dtype = data.dtype.type if data.dtype in (np.float64, np.float32) else None
        if dtype is None:
            raise TypeError("Storage holds float64 or float32 fields only")
        if data.ndim not in (1, 3):
            raise ValueError("Storage buffers are rank 1 or rank 3")
        self.data = data
        self.halo = int(halo)
        self.dtype = np.dtype(dtype)
        self.rank = data.ndim
        if self.rank == 3:
            szk, szj, pitch = data.shape
            self.szi = pitch if nx is None else int(nx) + 2 * self.halo
            if self.szi > pitch:
                raise ValueError("logical i extent exceeds the row pitch")
            self.pitch = pitch
        else:
            self.szi = data.shape[0]
            self.pitch = data.shape[0]
        self._memref = None

    # -- construction ------------------------------------------------------------------
    @classmethod
    def allocate3d(cls, nx, ny, nz, halo, dtype=np.float64, device="cpu", pitch_multiple=1, fill=0.0):
        """allocateStorage(sizes3D) of include/util.h:126-141, on `device`."""
        szi = nx + 2 * halo
        pitch = -(-szi // pitch_multiple) * pitch_multiple
        shape = (nz + 2 * halo, ny + 2 * halo, pitch)
        if device in ("host", "numpy"):
            buf = np.full(shape, fill, dtype=dtype)
        else:
            tdt = torch.float64 if np.dtype(dtype) == np.float64 else torch.float32
            buf = torch.full(shape, fill, dtype=tdt, device=device)
        return cls(buf, halo, nx=nx)

    @classmethod
    def allocate1d(cls, n, halo, dtype=np.float64, device="cpu", fill=0.0):
        """allocateStorage(size) of include/util.h:99-109, on `device`."""
        shape = (n + 2 * halo,)
        if device in ("host", "numpy"):
            return cls(np.full(shape, fill, dtype=dtype), halo)
        tdt = torch.float64 if np.dtype(dtype) == np.float64 else torch.float32
        return cls(torch.full(shape, fill, dtype=tdt, device=device), halo)

    # -- descriptor ----------------------------------------------------------------------
    @property
    def is_cuda(self) -> bool:
        return _is_torch(self.data) and self.data.is_cuda

    def data_ptr(self) -> int:
        return self.data.data_ptr() if _is_torch(self.data) else self.data.ctypes.data

    def memref(self):
        """The descriptor as a ctypes structure (kept alive by this object)."""
        ptr = self.data_ptr()
        h = self.halo
        if self.rank == 3:
            szk, szj, pitch = self.data.shape
            m = Memref3d(ptr, ptr, h * szj * pitch + h * pitch + h, (szk, szj, self.szi), (szj * pitch, pitch, 1))
        else:
            m = Memref1d(ptr, ptr, h, (self.data.shape[0],), (1,))
        self._memref = m
        return m

    # -- views ---------------------------------------------------------------------------
    def box(self, reach=(0, 0, 0, 0, 0, 0), nx=None, ny=None, nz=None):
        """View of [-ilo, nx+ihi) x [-jlo, ny+jhi) x [-klo, nz+khi), indexed [k, j, i]."""
        h = self.halo
        if self.rank == 1:
            n = self.data.shape[0] - 2 * h if ny is None else ny
            return self.data[h - reach[2]:h + n + reach[3]]
        szk, szj, _ = self.data.shape
        nx = self.szi - 2 * h if nx is None else nx
        ny = szj - 2 * h if ny is None else ny
        nz = szk - 2 * h if nz is None else nz
        ilo, ihi, jlo, jhi, klo, khi = reach
        return self.data[h - klo:h + nz + khi, h - jlo:h + ny + jhi, h - ilo:h + nx + ihi]

    def interior(self):
        return self.box()

    def numpy(self) -> np.ndarray:
        d = self.data
        return d.detach().cpu().numpy() if _is_torch(d) else d

    def __repr__(self):
        where = "cuda" if self.is_cuda else "host"
        return "Storage(rank=%d, shape=%s, halo=%d, %s, %s)" % (self.rank, tuple(self.data.shape), self.halo,
                                                                self.dtype.name, where)


def as_storage(x, halo: Optional[int] = None) -> Storage:
    if isinstance(x, Storage):
        return x
    if halo is None:
        raise ValueError("a raw buffer needs an explicit halo")
    return Storage(x, halo)


def same_layout(fields) -> Tuple[int, int]:
    """(row pitch, rows per plane) shared by rank-3 fields of one call."""
    lay = {(f.data.shape[1], f.pitch) for f in fields if f.rank == 3}
    if len(lay) > 1:
        raise ValueError("the rank-3 fields of one call must share their strides: %s" % sorted(lay))
    return next(iter(lay))
