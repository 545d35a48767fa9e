"""The tcgen05 tile of the learned preconditioner's convolutions: D = A B^T
with BF16 operands staged in the canonical no-swizzle K-major layout and FP32
accumulation in tensor memory.  Inputs are multiples of 1/4 in [-4, 4], so
every product and partial sum is exact in FP32: bit-exact against numpy."""
import ctypes as C

import numpy as np
import pytest

import xflow_gb300 as xf
from xflow_gb300 import capi

pytestmark = pytest.mark.gpu


def bf16_bits(a):
    """FP32 values exactly representable in BF16 -> their 16-bit patterns."""
    a = np.ascontiguousarray(a, np.float32)
    return (a.view(np.uint32) >> 16).astype(np.uint16)


@pytest.fixture(scope="module")
def ctx():
    c = xf.Context(0)
    yield c
    c.close()


def run(ctx, A, B, variant):
    N, K = B.shape
    D = np.zeros((128, N), np.float32)
    a, b = bf16_bits(A), bf16_bits(B)
    st = capi.lib().xf_tc_gemm_bf16(ctx.h, N, K, a.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p),
                                    D.ctypes.data_as(C.c_void_p), variant)
    xf._check(ctx.h, st)
    return D


@pytest.mark.parametrize("N,K", [(16, 16), (32, 48), (64, 64), (16, 256), (256, 32)])
def test_tc_gemm_exact(ctx, N, K):
    rng = np.random.Generator(np.random.PCG64(N * 1000 + K))
    A = rng.integers(-16, 17, (128, K)).astype(np.float32) / 4
    B = rng.integers(-16, 17, (N, K)).astype(np.float32) / 4
    want = (A.astype(np.float64) @ B.astype(np.float64).T).astype(np.float32)
    got = run(ctx, A, B, 0)
    np.testing.assert_array_equal(got, want)


def test_tc_gemm_layout_check(ctx):
    """Swapping the two core-matrix strides changes the result whenever K > 8
    and M > 8 (the descriptors' fields are not interchangeable)."""
    rng = np.random.Generator(np.random.PCG64(7))
    A = rng.integers(-16, 17, (128, 32)).astype(np.float32) / 4
    B = rng.integers(-16, 17, (32, 32)).astype(np.float32) / 4
    want = A @ B.T
    assert not np.array_equal(run(ctx, A, B, 1), want)
