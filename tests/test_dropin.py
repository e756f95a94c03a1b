"""The C++ drop-in headers (include/oeb/<k>.h) in place of the reference's kernels/<k>.h.

* CPU: the reference's own drivers (src/<k>.cpp), unmodified, compile and link against the
  drop-in headers and liboeb_gb300.so (skipped where the reference source tree is absent).
* GPU: tests/dropin/dropin_driver.cpp -- a driver in the reference's style -- calls all ten
  kernel functions through the drop-in headers on host fields (and on device fields for
  laplace) and checks every output bit for bit against the oracle.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

KERNELS = ("laplace", "hdiffsa", "hdiffsmag", "hadvuv", "hadvuv5th", "fastwavesuv", "uvbke", "nh_p_grad",
           "p_grad_c", "fvtp2d")
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def _cxx():
    return os.environ.get("CXX", "g++")


@pytest.mark.parametrize("name", KERNELS)
def test_reference_drivers_build_against_dropin_headers(pkg, orc, tmp_path, name):
    from oracle import build as ob
    ref = ob.reference_dir()
    if not (ref / "src" / ("%s.cpp" % name)).exists():
        pytest.skip("reference source tree absent")
    lib_dir = pkg.LIB_PATH.parent
    cmd = [_cxx(), "-std=c++17", "-O1", "-w", "-I", str(ROOT / "include" / "oeb"), "-I", str(ref / "include"),
           str(ref / "src" / ("%s.cpp" % name)), "-L", str(lib_dir), "-loeb_gb300",
           "-Wl,-rpath," + str(lib_dir), "-o", str(tmp_path / name)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr


@pytest.mark.gpu
def test_dropin_driver_matches_oracle_on_gpu(pkg, orc, tmp_path):
    from oracle import build as ob
    oracle_so = ob.build_oracle()
    lib_dir = pkg.LIB_PATH.parent
    exe = tmp_path / "dropin_driver"
    cmd = [_cxx(), "-std=c++17", "-O1", "-I", str(ROOT / "include" / "oeb"), "-I", str(ROOT / "tests" / "dropin"),
           "-I", str(CUDA / "include"), str(ROOT / "tests" / "dropin" / "dropin_driver.cpp"),
           "-L", str(lib_dir), "-loeb_gb300", "-L", str(oracle_so.parent), "-l:" + oracle_so.name,
           "-L", str(CUDA / "lib64"), "-lcudart",
           "-Wl,-rpath," + ":".join([str(lib_dir), str(oracle_so.parent), str(CUDA / "lib64")]), "-o", str(exe)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(run.stdout)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "PASSED" in run.stdout
