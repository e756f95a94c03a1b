"""The FP64 multiply, division, addition, subtraction and square root of the FP64 kernels,
done on the integer pipe, against the FP64 instructions.

oeb_selftest_fp64 computes seeded random operand pairs both ways on the GPU and counts
results that differ in any bit.  Eight distributions: any bit pattern (NaN, infinities,
zeros and subnormals take the fallback), ordinary magnitudes, exponents near both ends of
the normal range (results that underflow or overflow), short significands (rounding ties),
significands near all-ones and near zero (carries out of the significand), exact quotients
(b times a small integer, over b) and exact squares, cancellation (a and -a (1 + small)) and every alignment
shift of an addition (a and a 2^-k with changed low bits).
"""
from __future__ import annotations

import ctypes
import os

import pytest

pytestmark = pytest.mark.gpu

# 2^26 seeded pairs per case by default; OEB_SELFTEST_PAIRS raises it (e.g. 2^30 = 1073741824,
# about a minute a case) for a longer search of the operand space
PAIRS = int(os.environ.get("OEB_SELFTEST_PAIRS", 1 << 26))


@pytest.mark.parametrize("mode", range(8), ids=["any-bits", "ordinary", "range-ends", "ties", "carries", "exact",
                                                 "cancel", "align"])
@pytest.mark.parametrize("op", [0, 1, 2, 3, 4], ids=["mul", "div", "add", "sub", "sqrt"])
def test_integer_pipe_operation_is_the_fp64_operation(pkg, cuda, op, mode):
    lib = pkg.load_library()
    bad = ctypes.c_uint64(0)
    first = (ctypes.c_uint64 * 4)()
    st = lib.oeb_selftest_fp64(ctypes.c_int(op), ctypes.c_int64(PAIRS), ctypes.c_uint64(0xC0FFEE + 7919 * mode + op),
                               ctypes.c_int(mode), ctypes.byref(bad), first)
    assert st == 0, st
    assert bad.value == 0, "%d of %d results differ; first a=%016x b=%016x fp64=%016x int=%016x" % (
        bad.value, PAIRS, first[0], first[1], first[2], first[3])


def test_selftest_rejects_bad_arguments(pkg, cuda):
    lib = pkg.load_library()
    bad = ctypes.c_uint64(0)
    args = (ctypes.c_int64(16), ctypes.c_uint64(1))
    assert lib.oeb_selftest_fp64(ctypes.c_int(0), *args, ctypes.c_int(9), ctypes.byref(bad), None) != 0
    assert lib.oeb_selftest_fp64(ctypes.c_int(5), *args, ctypes.c_int(0), ctypes.byref(bad), None) != 0
    assert lib.oeb_selftest_fp64(ctypes.c_int(0), *args, ctypes.c_int(0), None, None) != 0


def test_fp64_add_rate_probe(pkg, cuda):
    # the FP64 pipe's rate, which bench.py's FP64-pipe roofline divides by: on a GB300 it is
    # about 1.6 additions a clock per SM (152 SMs, up to 2.07 GHz), far below the FP32 rate
    lib = pkg.load_library()
    rate, adds = ctypes.c_double(0.0), ctypes.c_double(0.0)
    assert lib.oeb_probe_fp64_add_rate(ctypes.byref(rate), ctypes.byref(adds)) == 0
    import torch
    sms = torch.cuda.get_device_properties(cuda).multi_processor_count
    per_clk_at_max = rate.value / (sms * 2.07e9)
    assert adds.value > 1e9 and 0.5 <= per_clk_at_max <= 64.0, (rate.value, per_clk_at_max)
    assert lib.oeb_probe_fp64_add_rate(None, None) != 0


def test_fp64_op_rate_probe(pkg, cuda):
    # the FP64 rate of each operation the stencils use; the addition agrees with the addition
    # probe, and the division and square root (instruction sequences) are slower
    lib = pkg.load_library()
    rates = []
    for op in range(5):
        r, n = ctypes.c_double(0.0), ctypes.c_double(0.0)
        assert lib.oeb_probe_fp64_rate(ctypes.c_int(op), ctypes.byref(r), ctypes.byref(n)) == 0
        assert r.value > 1e9 and n.value > 1e8, (op, r.value, n.value)
        rates.append(r.value)
    add = ctypes.c_double(0.0)
    assert lib.oeb_probe_fp64_add_rate(ctypes.byref(add), None) == 0
    assert 0.75 <= rates[0] / add.value <= 1.33, (rates[0], add.value)
    assert rates[3] < rates[0] and rates[4] < rates[0], rates
    assert lib.oeb_probe_fp64_rate(ctypes.c_int(5), ctypes.byref(add), None) == 12
    assert lib.oeb_probe_fp64_rate(ctypes.c_int(0), None, None) == 1


def test_probe_shuffle_neighbours(pkg, cuda):
    # both forms of each probe stencil give the same bits; the four launch times are measured
    lib = pkg.load_library()
    us = (ctypes.c_double * 4)()
    bad = (ctypes.c_uint64 * 2)()
    assert lib.oeb_probe_shuffle_neighbours(us, bad) == 0
    assert list(bad) == [0, 0]
    assert all(0.5 < t < 10000.0 for t in us), list(us)
    assert lib.oeb_probe_shuffle_neighbours(None, None) != 0
