"""The tensor-core building blocks (tcgen05 MMA over BF16 operands in
shared memory, FP32 accumulation in tensor memory) against plain
arithmetic on the same BF16 values."""
import ctypes as C

import numpy as np
import pytest

from mapp4py_gb300 import _lib

pytestmark = pytest.mark.gpu


def to_bf16(a):
    """Round float32 to bfloat16 (nearest even); returns the 16-bit patterns."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def from_bf16(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


def test_tc_gemm_matches_plain_product():
    rng = np.random.default_rng(0)
    for trial in range(2):
        A = to_bf16(rng.normal(size=(128, 64)))
        Bt = to_bf16(rng.normal(size=(64, 64)))
        D = np.zeros((128, 64), dtype=np.float32)
        _lib.check(_lib.load().mappg_tc_gemm_check(A.ctypes.data_as(C.c_void_p), Bt.ctypes.data_as(C.c_void_p),
                                                   D.ctypes.data_as(C.c_void_p)))
        ref = from_bf16(A).astype(np.float64) @ from_bf16(Bt).astype(np.float64).T
        assert np.max(np.abs(D - ref)) < 1e-4, np.max(np.abs(D - ref))
