"""Parity of the CUDA stencils with the oracle, through the C ABI, on the GPU.

FP64 results must be bit-identical to the oracle (the C restatement of the reference's
``_openmp`` kernels, itself pinned bit-exact to the reference in
test_oracle_vs_reference.py): the FP64 kernels are compiled without FP contraction and
IEEE division and square root round identically on both sides.  Every output buffer is
compared whole, so cells outside the written box must also keep their pre-call value.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_bitwise_equal

pytestmark = pytest.mark.gpu

H = 3
KERNELS = ("laplace", "hdiffsa", "hdiffsmag", "hadvuv", "hadvuv5th", "fastwavesuv", "uvbke", "nh_p_grad",
           "p_grad_c", "fvtp2d")


def _run_both(pkg, fields, orc, cuda, name, nx, ny, nz, seed, workload="physical", halo=H, pitch_multiple=1,
              scalars=None):
    import torch
    spec = pkg.KERNELS[name]
    inputs = fields.make_inputs(name, nx, ny, nz, seed=seed, workload=workload, halo=halo)
    sc = scalars if scalars is not None else fields.make_scalars(name, seed=seed)
    outs = fields.make_outputs(name, nx, ny, nz, halo=halo)
    want = {k: v.copy() for k, v in {**inputs, **outs}.items()}
    orc.run_oracle(spec, want, sc, nx, ny, nz, halo)
    dev = {}
    for k, v in {**inputs, **outs}.items():
        if v.ndim == 3 and pitch_multiple > 1:
            st = pkg.Storage.allocate3d(nx, ny, nz, halo, device=cuda, pitch_multiple=pitch_multiple)
            st.data[:, :, :v.shape[2]] = torch.from_numpy(v).to(cuda)
            dev[k] = st
        else:
            dev[k] = pkg.Storage(torch.from_numpy(v).to(cuda), halo, nx=nx if v.ndim == 3 else None)
    pkg.call(name, dev, sc, domain=(nx, ny, nz))
    torch.cuda.synchronize()
    for a in spec.by_role("out3"):
        got = dev[a.name].numpy()[:, :, :nx + 2 * halo]
        assert_bitwise_equal(np.ascontiguousarray(got), want[a.name], "%s.%s" % (name, a.name))


@pytest.mark.parametrize("name", KERNELS)
def test_small_nonsquare(pkg, fields, orc, cuda, name):
    _run_both(pkg, fields, orc, cuda, name, 40, 36, 5, seed=3)


@pytest.mark.parametrize("name", KERNELS)
def test_tiny_domain(pkg, fields, orc, cuda, name):
    _run_both(pkg, fields, orc, cuda, name, 1, 1, 1, seed=4)


@pytest.mark.parametrize("name", KERNELS)
def test_ragged_multitile_fronts(pkg, fields, orc, cuda, name):
    _run_both(pkg, fields, orc, cuda, name, 70, 97, 9, seed=5, workload="fronts")


@pytest.mark.parametrize("name", KERNELS)
def test_halo4_padded_pitch(pkg, fields, orc, cuda, name):
    # the reference drivers' halo of 4 (src/<k>.cpp:6) and rows padded to 16 elements
    _run_both(pkg, fields, orc, cuda, name, 33, 31, 4, seed=6, halo=4, pitch_multiple=16)


@pytest.mark.parametrize("name", ("laplace", "hdiffsa"))
def test_config_64x64x60_smooth(pkg, fields, orc, cuda, name):
    _run_both(pkg, fields, orc, cuda, name, 64, 64, 60, seed=0, workload="smooth")


@pytest.mark.parametrize("name", KERNELS)
def test_config_128x128x80(pkg, fields, orc, cuda, name):
    _run_both(pkg, fields, orc, cuda, name, 128, 128, 80, seed=1)


@pytest.mark.parametrize("name", KERNELS)
def test_driver_scalars(pkg, fields, orc, cuda, name):
    # the reference drivers' own scalar values (src/<k>.cpp)
    _run_both(pkg, fields, orc, cuda, name, 48, 48, 6, seed=7, scalars=fields.make_scalars(name, 7, "driver"))


@pytest.fixture(params=["direct", "staged", "async"])
def host_mode(request, pkg):
    """The host entry points in place on the host fields (where the device can address
    them), staged through device memory, and asynchronous (staged, returning once enqueued:
    the test synchronises before it reads the outputs)."""
    lib = pkg.load_library()
    assert lib.oeb_set_host_direct(1 if request.param == "direct" else 0) == 0
    assert lib.oeb_set_host_async(1 if request.param == "async" else 0) == 0
    yield request.param
    lib.oeb_set_host_direct(1)
    lib.oeb_set_host_async(0)


@pytest.mark.parametrize("name", KERNELS)
@pytest.mark.parametrize("size", [(37, 29, 4), (128, 96, 24)], ids=["37x29x4", "128x96x24"])
@pytest.mark.parametrize("memory", ["pageable", "pinned"])
def test_host_entry_points(pkg, fields, orc, host_mode, name, size, memory):
    """oeb_<k>_f64_host with host buffers: same bits, untouched cells preserved.  The larger
    case runs the staged copy / compute / copy pipeline over several k-slabs."""
    import torch
    spec = pkg.KERNELS[name]
    nx, ny, nz = size
    inputs = fields.make_inputs(name, nx, ny, nz, seed=8)
    sc = fields.make_scalars(name, seed=8)
    outs = fields.make_outputs(name, nx, ny, nz)
    want = {k: v.copy() for k, v in {**inputs, **outs}.items()}
    orc.run_oracle(spec, want, sc, nx, ny, nz, H)
    if memory == "pinned":
        host = {k: pkg.Storage(torch.from_numpy(v.copy()).pin_memory(), H) for k, v in {**inputs, **outs}.items()}
    else:
        host = {k: pkg.Storage(v.copy(), H) for k, v in {**inputs, **outs}.items()}
    pkg.call(name, host, sc, domain=(nx, ny, nz))
    torch.cuda.synchronize()  # an asynchronous call completes with its stream
    for a in spec.by_role("out3"):
        assert_bitwise_equal(host[a.name].numpy(), want[a.name], "%s.%s (host path)" % (name, a.name))
    for a in spec.by_role("in3"):
        assert_bitwise_equal(host[a.name].numpy(), inputs[a.name], "%s.%s input unchanged" % (name, a.name))


def test_reference_named_api(pkg, fields, orc, cuda):
    """The reference-named functions and their variants, with the module's domain globals."""
    import torch
    k = pkg.kernels
    old = (k.domain_size, k.domain_height)
    k.domain_size, k.domain_height = 24, 3
    try:
        inputs = fields.make_inputs("hdiffsa", 24, 24, 3, seed=9)
        outs = fields.make_outputs("hdiffsa", 24, 24, 3)
        want = {n: v.copy() for n, v in {**inputs, **outs}.items()}
        orc.run_oracle(pkg.KERNELS["hdiffsa"], want, {}, 24, 24, 3, H)
        for variant in ("hdiffsa", "hdiffsa_fullfusion", "hdiffsa_partialfusion", "hdiffsa_openmp"):
            d = {n: pkg.Storage(torch.from_numpy(v).to(cuda), H) for n, v in {**inputs, **outs}.items()}
            getattr(k, variant)(d["out"], d["in"], d["mask"], d["crlato"], d["crlatu"])
            torch.cuda.synchronize()
            assert_bitwise_equal(d["out"].numpy(), want["out"], variant)
    finally:
        k.domain_size, k.domain_height = old


def test_launches_are_counted(pkg, fields, cuda):
    import torch
    lib = pkg.load_library()
    before = lib.oeb_launch_count()
    inputs = fields.make_inputs("laplace", 16, 16, 2, seed=1)
    outs = fields.make_outputs("laplace", 16, 16, 2)
    d = {n: pkg.Storage(torch.from_numpy(v).to(cuda), H) for n, v in {**inputs, **outs}.items()}
    pkg.call("laplace", d, {}, domain=(16, 16, 2))
    torch.cuda.synchronize()
    assert lib.oeb_launch_count() == before + 1


@pytest.mark.parametrize("kb", [2, 3, 8])
def test_kblock_does_not_change_results(pkg, fields, orc, cuda, kb):
    # oeb_set_kblock changes how the k-levels are split among CTAs, never a result
    lib = pkg.load_library()
    assert lib.oeb_set_kblock(kb) == 0
    try:
        for name in KERNELS:
            _run_both(pkg, fields, orc, cuda, name, 40, 36, 7, seed=13)
    finally:
        lib.oeb_set_kblock(0)


@pytest.mark.parametrize("shape", [1, 2], ids=["32x8", "64x16"])
def test_tile_shape_does_not_change_results(pkg, fields, orc, cuda, shape):
    # oeb_set_tile_shape changes the tiles of the advection stencils (forward bit-exact with
    # the oracle; ragged tiles on every edge), never a result
    lib = pkg.load_library()
    assert lib.oeb_set_tile_shape(shape) == 0
    try:
        for name in ("hadvuv", "hadvuv5th"):
            _run_both(pkg, fields, orc, cuda, name, 70, 41, 5, seed=15)
    finally:
        lib.oeb_set_tile_shape(0)
    assert lib.oeb_set_tile_shape(3) != 0 and lib.oeb_set_tile_shape(-1) != 0


@pytest.mark.parametrize("shape", [1, 2], ids=["32x8", "64x16"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_tile_shape_adjoint_bits(pkg, fields, cuda, shape, dtype):
    # the advection adjoints (their terms kernel takes the tile shape) give the same bits in
    # every shape
    import torch
    lib = pkg.load_library()
    nx, ny, nz = 70, 41, 5
    for name in ("hadvuv", "hadvuv5th"):
        spec = pkg.KERNELS[name]
        x = fields.make_inputs(name, nx, ny, nz, seed=16)
        sc = fields.make_scalars(name, seed=16)
        rng = np.random.default_rng(16)
        yb = {n: rng.normal(size=x["uin"].shape) for n in spec.semantic_outputs}

        def dev(a):
            t = torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to(cuda)
            return pkg.Storage(t, H, nx=nx if t.ndim == 3 else None)

        def adj():
            xb = {n: dev(np.zeros_like(x["uin"])) for n in pkg.ACTIVE[name]}
            pkg.adjoint(name, {k: dev(v) for k, v in x.items()}, {k: dev(v) for k, v in yb.items()}, xb, sc,
                        domain=(nx, ny, nz))
            torch.cuda.synchronize()
            return {k: v.numpy() for k, v in xb.items()}

        want = adj()
        assert lib.oeb_set_tile_shape(shape) == 0
        try:
            got = adj()
        finally:
            lib.oeb_set_tile_shape(0)
        for n in want:
            assert_bitwise_equal(got[n], want[n], "%s adjoint %sb shape %d" % (name, n, shape))


@pytest.mark.parametrize("slabs", [2, 3, 8])
def test_host_slabs_do_not_change_results(pkg, fields, orc, slabs):
    # the staged host path over 2, 3 and 8 k-slabs (7 levels: uneven slabs)
    lib = pkg.load_library()
    assert lib.oeb_set_host_direct(0) == 0 and lib.oeb_set_host_slabs(slabs) == 0
    try:
        for name in KERNELS:
            spec = pkg.KERNELS[name]
            nx, ny, nz = 33, 30, 7
            inputs = fields.make_inputs(name, nx, ny, nz, seed=14)
            sc = fields.make_scalars(name, seed=14)
            outs = fields.make_outputs(name, nx, ny, nz)
            want = {k: v.copy() for k, v in {**inputs, **outs}.items()}
            orc.run_oracle(spec, want, sc, nx, ny, nz, H)
            host = {k: pkg.Storage(v.copy(), H) for k, v in {**inputs, **outs}.items()}
            pkg.call(name, host, sc, domain=(nx, ny, nz))
            for a in spec.by_role("out3"):
                assert_bitwise_equal(host[a.name].numpy(), want[a.name], "%s.%s slabs %d" % (name, a.name, slabs))
    finally:
        lib.oeb_set_host_slabs(0)
        lib.oeb_set_host_direct(1)


def test_async_host_calls_pipeline(pkg, fields, orc, cuda):
    """All ten host entry points enqueued asynchronously on one stream, back to back (each
    call's copy-in overlaps the previous calls' compute and copy-out), one synchronisation at
    the end: every output as the oracle's, every input unchanged."""
    import torch
    lib = pkg.load_library()
    nx, ny, nz = 70, 53, 9
    stream = torch.cuda.Stream()
    cases = {}
    for name in KERNELS:
        spec = pkg.KERNELS[name]
        inputs = fields.make_inputs(name, nx, ny, nz, seed=21)
        sc = fields.make_scalars(name, seed=21)
        outs = fields.make_outputs(name, nx, ny, nz)
        want = {k: v.copy() for k, v in {**inputs, **outs}.items()}
        orc.run_oracle(spec, want, sc, nx, ny, nz, H)
        host = {k: pkg.Storage(torch.from_numpy(v.copy()).pin_memory(), H) for k, v in {**inputs, **outs}.items()}
        cases[name] = (spec, inputs, sc, want, host)
    assert lib.oeb_set_host_async(1) == 0
    try:
        for name, (spec, inputs, sc, want, host) in cases.items():
            pkg.call(name, host, sc, domain=(nx, ny, nz), stream=stream)
        stream.synchronize()
    finally:
        lib.oeb_set_host_async(0)
    for name, (spec, inputs, sc, want, host) in cases.items():
        for a in spec.by_role("out3"):
            assert_bitwise_equal(host[a.name].numpy(), want[a.name], "%s.%s (asynchronous host path)" % (name, a.name))
        for a in spec.by_role("in3"):
            assert_bitwise_equal(host[a.name].numpy(), inputs[a.name], "%s.%s input unchanged" % (name, a.name))
