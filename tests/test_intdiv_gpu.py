"""The FP64 path's IEEE division and square root run on the integer pipe (cato_intdiv.cuh).
cato_gpu_check_divsqrt sends 2^30 seeded operand pairs through them and through the hardware
instructions on the GPU; every case the integer routines take must agree in every bit.  It also
measures the hardware FP32 approximations that seed the routines over all their inputs: they must
stay within the 8 ulps for which tests/intdiv_check.cpp verifies the routines on the host."""
import ctypes

import pytest

from fvleg_2d_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 0x5eed])
def test_device_division_and_sqrt_bit_exact(seed):
    L = _lib.load(build_if_missing=True)
    tested = (ctypes.c_uint64 * 2)()
    bad = (ctypes.c_uint64 * 2)()
    ulps = (ctypes.c_int32 * 2)()
    assert L.cato_gpu_check_divsqrt(1 << 30, seed, tested, bad, ulps) == 0
    assert (bad[0], bad[1]) == (0, 0)
    assert 0 <= ulps[0] <= 8 and 0 <= ulps[1] <= 8, (ulps[0], ulps[1])
    # random bit patterns include zeros, subnormals, inf and NaN (hardware fallback), so fewer
    # than all 2^30 cases take the integer routines
    assert tested[0] > (1 << 29) and tested[1] > (1 << 29)


def test_check_rejects_bad_arguments():
    L = _lib.load(build_if_missing=True)
    tested = (ctypes.c_uint64 * 2)()
    bad = (ctypes.c_uint64 * 2)()
    ulps = (ctypes.c_int32 * 2)()
    assert L.cato_gpu_check_divsqrt(-1, 0, tested, bad, ulps) != 0
    assert L.cato_gpu_check_divsqrt(0, 0, tested, bad, ulps) == 0
    assert (tested[0], tested[1], bad[0], bad[1]) == (0, 0, 0, 0)
    assert ulps[0] >= 0 and ulps[1] >= 0
