"""Build recipe for the CPU oracle (TEST INFRASTRUCTURE).

Two shared libraries, both compiled with plain gcc/g++ (no make, no cmake), so the
recipe runs the same way on an x86 host and on an aarch64 GPU host:

* ``oracle/_build/liboeb_oracle.so`` -- the C restatement in ``oeb_oracle.c``;
  built wherever ``build()`` runs.
* ``oracle/_ref/liboeb_ref.so`` -- the reference's own ``include/util.h`` and
  ``kernels/*.h``, compiled from where they lie in the reference source tree through
  the harness TUs in ``oracle/ref/`` (nothing is copied).  Built only when that
  source tree is present (``OEB_REFERENCE_DIR``, else a ``reference`` directory beside
  this repository's root).

Both use ``-O3 -fopenmp`` (the reference's CMakeLists.txt:12 flags plus its OpenMP
link) and ``-ffp-contract=off``: x86-64 gcc emits no FMA by default, but aarch64 gcc
contracts a*b+c unless told not to, which would change the last bits.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
BUILD_DIR = HERE / "_build"
REF_DIR = HERE / "_ref"
ORACLE_SO = BUILD_DIR / "liboeb_oracle.so"
REF_SO = REF_DIR / "liboeb_ref.so"
REF_KERNELS = ("laplace", "hdiffsa", "hdiffsmag", "hadvuv", "hadvuv5th", "fastwavesuv", "uvbke",
               "nh_p_grad", "p_grad_c", "fvtp2d")
COMMON_FLAGS = ["-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"]


def reference_dir() -> Path:
    """The reference source tree: $OEB_REFERENCE_DIR, else ``reference`` beside the repository."""
    env = os.environ.get("OEB_REFERENCE_DIR")
    return Path(env) if env else REPO.parent / "reference"


def _newer(target: Path, sources) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(Path(s).stat().st_mtime <= t for s in sources)


def _run(cmd, cwd=None):
    proc = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(map(str, cmd)), proc.stdout, proc.stderr))


def build_oracle(force: bool = False) -> Path:
    srcs = [HERE / "oeb_oracle.c", HERE / "oracle_impl.h", REPO / "include" / "oeb_gb300.h"]
    if not force and _newer(ORACLE_SO, srcs):
        return ORACLE_SO
    BUILD_DIR.mkdir(exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    tmp = ORACLE_SO.with_suffix(".so.tmp")
    _run([cc, "-std=c11", *COMMON_FLAGS, "-o", str(tmp), str(HERE / "oeb_oracle.c"), "-lm"])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference headers into oracle/_ref/liboeb_ref.so; None if absent."""
    ref = reference_dir()
    if not (ref / "include" / "util.h").exists():
        return None
    srcs = [HERE / "ref" / f"ref_{k}.cpp" for k in REF_KERNELS]
    deps = srcs + [HERE / "ref" / "ref_common.hpp"] + [ref / "kernels" / f"{k}.h" for k in REF_KERNELS]
    deps.append(ref / "include" / "util.h")
    if not force and _newer(REF_SO, deps):
        return REF_SO
    REF_DIR.mkdir(exist_ok=True)
    obj_dir = REF_DIR / "obj"
    obj_dir.mkdir(exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    inc = ["-I", str(ref / "include"), "-I", str(ref / "kernels")]

    def compile_one(src: Path) -> Path:
        obj = obj_dir / (src.stem + ".o")
        _run([cxx, "-std=c++17", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-w", *inc, "-c", str(src),
              "-o", str(obj)])
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = REF_SO.with_suffix(".so.tmp")
    _run([cxx, "-shared", "-fopenmp", "-o", str(tmp), *map(str, objs)])
    os.replace(tmp, REF_SO)
    shutil.rmtree(obj_dir, ignore_errors=True)
    return REF_SO


def build(force: bool = False):
    return build_oracle(force), build_ref(force)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
