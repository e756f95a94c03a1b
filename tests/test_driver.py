"""oeb_driver: the reference's ./<kernel> ALGO domain_size domain_height on the GPU.

The driver is a reference-style C++ program (open-earth-benchmarks_gb300/driver/) whose kernel
headers are the drop-in ones over device-resident fields.  Argument handling is checked on
the CPU (it fails before any CUDA call); the sweep of all ten kernels runs on the GPU.
"""
from __future__ import annotations

import json
import subprocess

import pytest

KERNELS = {"laplace", "hdiffsa", "hdiffsmag", "hadvuv", "hadvuv5th", "fastwavesuv", "uvbke", "nh_p_grad", "p_grad_c",
           "fvtp2d"}


@pytest.fixture(scope="module")
def driver(pkg):
    import importlib
    return str(importlib.import_module("oeb_gb300.build").build_driver())


def _run(driver, *args, timeout=300):
    return subprocess.run([driver, *args], capture_output=True, text=True, timeout=timeout)


def test_usage_errors(driver):
    for args in ([], ["laplace", "0", "32"], ["laplace", "--bogus"], ["laplace", "0", "0", "8"]):
        proc = _run(driver, *args)
        assert proc.returncode == 1 and "Usage" in proc.stderr, (args, proc.stdout, proc.stderr)


def test_unknown_algo_and_kernel(driver):
    # the reference's drivers print "Unknown ALGO" and exit normally (src/laplace.cpp:73-75)
    proc = _run(driver, "laplace", "7")
    assert proc.returncode == 0 and "Unknown ALGO" in proc.stdout
    proc = _run(driver, "fvtp2d", "2")  # fvtp2d has the default and fullfusion variants only
    assert proc.returncode == 0 and "Unknown ALGO" in proc.stdout
    proc = _run(driver, "nosuchkernel", "0")
    assert proc.returncode == 1 and "unknown kernel" in proc.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["", "--f32"])
def test_sweep_all_kernels_with_adjoint(driver, precision):
    args = ["all", "0", "48", "10", "--count", "3", "--json", "--adjoint"] + ([precision] if precision else [])
    proc = _run(driver, *args)
    assert proc.returncode == 0, proc.stdout + proc.stderr
    lines = proc.stdout.splitlines()
    recs = [json.loads(ln) for ln in lines if ln.startswith("{")]
    assert {r["kernel"] for r in recs} == KERNELS  # every stencil has an adjoint
    for r in recs:
        assert r["mode"] == "forward+adjoint" and r["count"] == 3
        assert r["precision"] == ("f32" if precision else "f64")
        assert r["ms_per_call"] > 0 and r["gpts"] > 0
    # the reference's timer line, labelled with the adjoint
    for name in KERNELS:
        assert [ln for ln in lines if ln.startswith("%s + adjoint: " % name) and ln.endswith(" ms")], name
    assert sum(1 for ln in lines if " + adjoint: " in ln) == len(KERNELS)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["", "--f32"])
@pytest.mark.parametrize("algo", ["0", "3"])
def test_sweep_all_kernels(driver, precision, algo):
    args = ["all", algo, "48", "10", "--count", "5", "--json"] + ([precision] if precision else [])
    proc = _run(driver, *args)
    assert proc.returncode == 0, proc.stdout + proc.stderr
    lines = proc.stdout.splitlines()
    assert lines[:3] == ["ALGO: %s" % algo, "domain_size: 48", "domain_height: 10"]
    recs = [json.loads(ln) for ln in lines if ln.startswith("{")]
    # fvtp2d has no openmp variant (ALGO 3): "Unknown ALGO", as in the reference
    want = KERNELS - {"fvtp2d"} if algo == "3" else KERNELS
    assert {r["kernel"] for r in recs} == want
    assert ("Unknown ALGO" in lines) == (algo == "3")
    for r in recs:
        assert r["precision"] == ("f32" if precision else "f64")
        assert r["domain"] == [48, 48, 10] and r["count"] == 5
        assert r["gpts"] > 0 and r["hbm_gbs"] > 0
        # the fraction of this GPU's copy rate, which the driver measures itself
        assert r["copy_gbs"] > 1000 and abs(r["hbm_frac_of_copy"] - r["hbm_gbs"] / r["copy_gbs"]) < 1e-3
        if precision:
            # FP32 against the FP64 run of the same variant on the same fills (the FP64 stencils are
            # the reference's arithmetic bit for bit): storage rounding of the drivers' analytic inputs
            assert 0.0 <= r["rms_rel_err_vs_f64"] <= r["max_rel_err_vs_f64"] < 1e-2, r
        else:
            assert "max_rel_err_vs_f64" not in r
    timer = [ln for ln in lines if " count, avg " in ln]
    assert len(timer) == len(want)


@pytest.mark.gpu
def test_single_kernel_reference_defaults(driver):
    # ./laplace with no arguments: ALGO 0, 64 x 64 x 60, the reference's count of 1000
    proc = _run(driver, "laplace")
    assert proc.returncode == 0, proc.stderr
    assert "laplace: " in proc.stdout and "/ 1000 count" in proc.stdout
