"""Builds liboeb_gb300.so, the sm_103a stencil library, in-tree.

One nvcc invocation per translation unit (run in parallel), then one link.  Only
``-gencode arch=compute_103a,code=sm_103a`` is emitted.  The FP64 translation units are
compiled with ``--fmad=false`` so that no multiply-add is contracted, which keeps every
FP64 result bit-identical to the reference compiled without FP contraction.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
REPO = PKG.parent
BUILD_DIR = PKG / "_build"
LIB = PKG / "liboeb_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
BASE_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-I", str(REPO / "include")]

# Translation units and their extra flags.
UNITS = {
    "abi_common.cu": [],
    "host_staging.cu": [],
    "k_pointwise.cu": ["--fmad=false"],
    "k_hdiff.cu": ["--fmad=false"],
    "k_fastwavesuv.cu": ["--fmad=false"],
    "k_fvtp2d.cu": ["--fmad=false"],
    "chain.cu": ["--fmad=false"],
    "batch.cu": [],
    "step.cu": ["--fmad=false"],
    "selftest.cu": [],
}

# Units compiled more than once, each time into an object of its own with extra flags: the
# step kernel for 2, 3 and 4 CTAs an SM.
VARIANTS = {"step.cu": [("step_c%d" % n, ["-DOEB_STEP_MIN_CTAS=%d" % n]) for n in (2, 3, 4)]}

# The stencil files step.cu compiles its bodies from.
STEP_INCLUDES = ("k_fastwavesuv.cu", "k_fvtp2d.cu", "k_hdiff.cu", "k_pointwise.cu", "chain.cu")


def nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def _run(cmd):
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("nvcc failed: %s\n%s\n%s" % (" ".join(cmd), proc.stdout, proc.stderr))
    return proc.stdout + proc.stderr


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    """Compile every unit that changed and link liboeb_gb300.so; returns its path."""
    BUILD_DIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [REPO / "include" / "oeb_gb300.h"]
    units = [u for u in UNITS if (CSRC / u).exists()]
    jobs = []
    objs = []
    for u in units:
        src = CSRC / u
        # step.cu includes the stencil files themselves (their bodies)
        extra = [CSRC / f for f in STEP_INCLUDES] if u == "step.cu" else []
        for stem, vflags in VARIANTS.get(u, [(src.stem, [])]):
            obj = BUILD_DIR / (stem + ".o")
            objs.append(obj)
            if force or _stale(obj, [src, *headers, *extra]):
                flags = BASE_FLAGS + UNITS[u] + vflags + (["-Xptxas", "-v"] if verbose_ptxas else [])
                jobs.append((stem, [nvcc(), *ARCH, *flags, "-c", str(src), "-o", str(obj)]))
    logs = {}
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for (u, _), out in zip(jobs, ex.map(lambda j: _run(j[1]), jobs)):
                logs[u] = out
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)])
        os.replace(tmp, LIB)
    if verbose_ptxas:
        for u, out in logs.items():
            sys.stderr.write("==== %s\n%s" % (u, out))
    return LIB


DRIVER_DIR = PKG / "driver"
DRIVER = PKG / "oeb_driver"
DRIVER_UNITS = ("oeb_driver_main.cpp", "oeb_driver_f64.cpp", "oeb_driver_f32.cpp")


def _cuda_home() -> Path:
    return Path(nvcc()).resolve().parent.parent if Path(nvcc()).exists() else Path("/usr/local/cuda")


def build_driver(force: bool = False) -> Path:
    """The GPU driver (driver/): a reference-style C++ program over the drop-in headers,
    linked against liboeb_gb300.so; returns its path."""
    lib = build()
    deps = [*(DRIVER_DIR / u for u in DRIVER_UNITS), *DRIVER_DIR.glob("*.h"), *DRIVER_DIR.glob("*.inc"),
            *(REPO / "include" / "oeb").glob("*"), REPO / "include" / "oeb_gb300.h", lib]
    if not force and not _stale(DRIVER, deps):
        return DRIVER
    cuda = _cuda_home()
    cxx = os.environ.get("CXX", "g++")
    tmp = DRIVER.with_suffix(".tmp")
    cmd = [cxx, "-std=c++17", "-O2", "-I", str(REPO / "include" / "oeb"), "-I", str(REPO / "include"), "-I",
           str(DRIVER_DIR), "-I", str(cuda / "include"), *(str(DRIVER_DIR / u) for u in DRIVER_UNITS), "-L", str(PKG),
           "-loeb_gb300", "-L", str(cuda / "lib64"), "-lcudart", "-Wl,-rpath," + str(PKG), "-o", str(tmp)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("driver build failed: %s\n%s" % (" ".join(cmd), proc.stderr))
    os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
