"""mappg_fp64_fma_rate: the FP64 roof that the FP64 path's kernels are read
against (GB300 runs FP64 far below its FP32 rate, so for those kernels the
arithmetic pipe, not HBM, is the bound).  The measured rate is finite and
positive, two measurements agree within a factor of two, and bad arguments
are refused."""
import ctypes as C
import math

import pytest

from mapp4py_gb300 import _lib

pytestmark = pytest.mark.gpu

ERR_ARG = -1  # MAPPG_ERR_ARG


def test_fp64_fma_rate_is_measured_and_repeatable():
    r1 = _lib.fp64_fma_rate(iters=2048, reps=3)
    r2 = _lib.fp64_fma_rate(iters=2048, reps=3)
    # TFLOP/s: far above zero, and far below any single GPU's FP64 rate
    # (a value beyond that would mean the timed kernel skipped its work)
    assert math.isfinite(r1) and 0.05 < r1 < 100.0
    assert 0.5 < r1 / r2 < 2.0
    t = C.c_double()
    L = _lib.load()
    assert L.mappg_fp64_fma_rate(0, 1, C.byref(t)) == ERR_ARG
    assert L.mappg_fp64_fma_rate(16, 0, C.byref(t)) == ERR_ARG
    assert L.mappg_fp64_fma_rate(16, 1, None) == ERR_ARG
