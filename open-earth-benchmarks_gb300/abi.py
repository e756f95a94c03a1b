"""ctypes binding of liboeb_gb300.so (the C ABI in include/oeb_gb300.h).

The library is the product: there is no fallback.  If it has not been built,
:func:`load_library` raises :class:`OebError` telling how to build it.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "liboeb_gb300.so"
HEADER = PKG.parent / "include" / "oeb_gb300.h"

OEB_OK = 0
STATUS_NAMES = {
    0: "OEB_OK", 1: "OEB_ERR_NULL", 2: "OEB_ERR_DOMAIN", 3: "OEB_ERR_LAYOUT", 4: "OEB_ERR_HALO",
    5: "OEB_ERR_ALIGNMENT", 6: "OEB_ERR_CUDA", 7: "OEB_ERR_ALLOC", 8: "OEB_ERR_ALIAS", 9: "OEB_ERR_UNSUPPORTED",
    10: "OEB_ERR_TIMEOUT", 11: "OEB_ERR_TOO_LARGE", 12: "OEB_ERR_ARGUMENT",
}


class OebError(RuntimeError):
    """A non-OK oeb_status, or the library missing."""

    def __init__(self, message, status=None):
        super().__init__(message)
        self.status = status


_lib = None
_lock = threading.Lock()


def load_library() -> ctypes.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise OebError("liboeb_gb300.so is not built (%s); run `python -c \"import __graft_entry__ as g; "
                               "g.build()\"` first" % LIB_PATH)
            lib = ctypes.CDLL(str(LIB_PATH))
            lib.oeb_status_string.restype = ctypes.c_char_p
            lib.oeb_status_string.argtypes = [ctypes.c_int]
            lib.oeb_last_cuda_error.restype = ctypes.c_char_p
            lib.oeb_launch_count.restype = ctypes.c_uint64
            lib.oeb_abi_version.restype = ctypes.c_int
            lib.oeb_memref3d_span_bytes_f64.restype = ctypes.c_int64
            lib.oeb_memref3d_span_bytes_f32.restype = ctypes.c_int64
            _lib = lib
    return _lib


def check(status: int, what: str = "oeb call") -> None:
    """Raise OebError for a non-OK status, with the library's description."""
    if status == OEB_OK:
        return
    lib = load_library()
    msg = lib.oeb_status_string(status).decode()
    if status == 6:  # OEB_ERR_CUDA
        msg += " (%s)" % lib.oeb_last_cuda_error().decode()
    raise OebError("%s failed: %s [%s]" % (what, msg, STATUS_NAMES.get(status, status)), status)


def declared_functions(header: Path = HEADER):
    """Names of every function declared in include/oeb_gb300.h."""
    import re
    text = header.read_text()
    return sorted(set(re.findall(r"^OEB_API\s+[A-Za-z0-9_ *]+?\b(oeb_[a-z0-9_]+)\(", text, flags=re.M)))


def entry(name: str):
    """The C function `name`, returning int (oeb_status)."""
    fn = getattr(load_library(), name)
    fn.restype = ctypes.c_int
    return fn
