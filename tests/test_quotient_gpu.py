"""The dequantisation quotient of every half-output epilogue (RN(1/d) and two
FMA correction steps, Markstein's method) against the IEEE division, bit for
bit, over every int32 numerator: the scales the attention path uses, powers
of two, the range edges and log-uniform random divisors."""
import numpy as np
import pytest
import torch

from magicube_gb300 import _lib

pytestmark = pytest.mark.gpu

_rng = np.random.default_rng(2026)
DIVISORS = ([60.0 ** 2, 36.0 ** 2, 127.0 ** 2, 44.26 ** 2, 36.0 * 32.0, 60.0 * 100.0, 1.0, 3.0, 7.0, 0.1, 1e-3,
             127.0 * 55.5 * 44.3, float(np.float32(np.float32(3600.0) / np.float32(0.125))),
             2.0 ** -60, 2.0 ** 60, 1.5 * 2.0 ** -60, 1.9 * 2.0 ** 59, 2.0 ** -61, 2.0 ** 61, -3600.0]
            + [float(2.0 ** x) for x in _rng.uniform(-60, 60, size=12)])


@pytest.mark.parametrize("d", DIVISORS)
def test_quotient_equals_ieee_division(cuda, d):
    lo, hi = -(2 ** 31), 2 ** 31
    counters = torch.tensor([0, hi], dtype=torch.int64, device=cuda)
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(_lib.probe_lib().mcCheckQuotients(float(d), lo, hi, counters.data_ptr(), stream), "mcCheckQuotients")
    bad, first = counters.tolist()
    assert bad == 0, f"{bad} mismatches, first numerator {first}"


@pytest.mark.parametrize("lo,hi", [(0x00000000, 0x4A800000), (0x80000000, 0xCA800000)])
def test_small_int_conversions_equal_hardware(cuda, lo, hi):
    """The add-and-reinterpret float-to-int of the dense-tile SDDMM epilogue
    equals cvt.rni (and the toward-zero form cvt.rzi) for every float with
    |f| < 2^22 (bit patterns up to 0x4A800000 = 2^22, both signs)."""
    counters = torch.tensor([0, -1], dtype=torch.int64, device=cuda)
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(_lib.probe_lib().mcCheckSmallIntConversions(lo, hi, counters.data_ptr(), stream), "mcCheckSmallIntConversions")
    bad, first = counters.tolist()
    assert bad == 0, f"{bad} mismatches, first pattern {first & 0xFFFFFFFFFFFFFFFF:#x}"
