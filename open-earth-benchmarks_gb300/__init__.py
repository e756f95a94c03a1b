"""GB300-native (sm_103a) open-earth-benchmarks stencils.

The ten weather/climate stencils of monellz/open-earth-benchmarks (laplace, hdiffsa,
hdiffsmag, hadvuv, hadvuv5th, fastwavesuv, uvbke, nh_p_grad, p_grad_c, fvtp2d) as
hand-written CUDA kernels behind a C ABI (include/oeb_gb300.h, liboeb_gb300.so), with the
reference's kernel functions mirrored by name (:mod:`.kernels`) and its strided field
descriptor mirrored by :class:`.storage.Storage`.

The directory name is not a Python identifier; load it with ``__graft_entry__.load_package()``
(registered as ``oeb_gb300``).
"""
from .abi import OebError, check, declared_functions, load_library, LIB_PATH
from .specs import ACTIVE, ADJ_FIELDS, KERNELS, KERNEL_NAMES, DRIVER_SCALARS
from .storage import Domain, Memref1d, Memref3d, Storage
from . import kernels
from .kernels import adjoint, call, tangent_linear, VARIANTS
from . import chain

__all__ = ["OebError", "check", "declared_functions", "load_library", "LIB_PATH", "KERNELS", "KERNEL_NAMES",
           "DRIVER_SCALARS", "ACTIVE", "ADJ_FIELDS", "tangent_linear", "adjoint", "Domain", "Memref1d", "Memref3d",
           "Storage", "kernels", "chain", "call", "VARIANTS"]
