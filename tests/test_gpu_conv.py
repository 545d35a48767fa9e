"""The tensor-core 3x3x3 convolution (implicit GEMM on tcgen05) against a
numpy FP64 convolution of the same BF16 inputs and weights.

Bars: FP32 output within 1e-5 x max|y| (FP32 accumulation of exact BF16
products in a different order); BF16 output within one BF16 rounding
(2^-8 relative) of the FP64 result.
"""
import ctypes as C

import numpy as np
import pytest

import xflow_gb300 as xf
from xflow_gb300 import capi

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx():
    c = xf.Context(0)
    yield c
    c.close()


def bf16_round(a):
    """Round FP32 to the nearest BF16 (ties to even), returned as FP32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def conv_ref(x, W, bias, mask, relu):
    """x [n1,n2,n3,ci], W [27,co,ci] -> [n1,n2,n3,co] in FP64 (cells outside the
    box read as 0)."""
    n1, n2, n3, ci = x.shape
    co = W.shape[1]
    xp = np.zeros((n1 + 2, n2 + 2, n3 + 2, ci))
    xp[1:-1, 1:-1, 1:-1] = x
    y = np.zeros((n1, n2, n3, co))
    for t in range(27):
        di, dj, dk = t // 9, (t // 3) % 3, t % 3
        y += xp[di:di + n1, dj:dj + n2, dk:dk + n3] @ W[t].astype(np.float64).T
    if bias is not None:
        y += bias
    if relu:
        y = np.maximum(y, 0)
    return y * mask[..., None]


def run_conv(ctx, x, W, bias, mask, relu, out_fp32, out_ch=None):
    """Activations in channel planes of 8 (plane q: channels 8q..8q+7 of every
    cell, each plane with its zero margins); FP32 output as cell rows."""
    n1, n2, n3, ci = x.shape
    co = W.shape[1]
    out_ch = co if out_ch is None else out_ch
    n = n1 * n2 * n3
    margin = n2 * n3 + n3 + 1 + 128
    rows = n + 2 * margin
    xb = torch.zeros((ci // 8, rows, 8), dtype=torch.bfloat16, device="cuda")
    planes = x.reshape(n, ci // 8, 8).transpose(1, 0, 2).astype(np.float32)
    xb[:, margin:margin + n] = torch.from_numpy(np.ascontiguousarray(planes)).to("cuda", torch.bfloat16)
    Wt = torch.from_numpy(W.astype(np.float32)).to("cuda", torch.bfloat16).contiguous()
    bt = torch.from_numpy(bias.astype(np.float32)).cuda() if bias is not None else None
    mt = torch.from_numpy(mask.reshape(n).astype(np.uint8)).cuda()
    if out_fp32:
        out = torch.zeros((n, out_ch), dtype=torch.float32, device="cuda")
        pitch = out_ch
    else:
        out = torch.zeros((out_ch // 8, n, 8), dtype=torch.bfloat16, device="cuda")
        pitch = n * 8
    torch.cuda.synchronize()
    st = capi.lib().xf_conv3d_bf16(ctx.h, n1, n2, n3, C.c_void_p(xb.data_ptr() + margin * 8 * 2), rows * 8, ci,
                                   C.c_void_p(Wt.data_ptr()), C.c_void_p(bt.data_ptr()) if bt is not None else None,
                                   co, C.c_void_p(mt.data_ptr()), C.c_void_p(out.data_ptr()), pitch, out_ch,
                                   int(out_fp32), int(relu))
    xf._check(ctx.h, st)
    xf._check(ctx.h, capi.lib().xf_conv_status(ctx.h))
    y = out.float().cpu().numpy()
    if not out_fp32:
        y = y.transpose(1, 0, 2).reshape(n, out_ch)
    return y.reshape(n1, n2, n3, out_ch)


def case(shape, ci, co, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    mask = np.zeros(shape)
    mask[1:-1, 1:-1, 1:-1] = 1
    mask *= rng.random(shape) > 0.1          # holes: inactive interior cells
    x = bf16_round(rng.standard_normal(shape + (ci,))) * mask[..., None]
    W = bf16_round(rng.standard_normal((27, co, ci)) / np.sqrt(27 * ci))
    bias = rng.standard_normal(co).astype(np.float32) * 0.1
    return x, W, bias, mask


# (32, 96) and (16, 128): 3 co > 256, the per-tap kernel (k_conv3_tc); the rest stack the k taps
@pytest.mark.parametrize("ci,co", [(16, 16), (16, 32), (32, 64), (96, 32), (48, 16), (32, 96), (16, 128)])
def test_conv_fp32_out(ctx, ci, co):
    x, W, bias, mask = case((10, 9, 12), ci, co, ci * 100 + co)
    for relu in (0, 1):
        got = run_conv(ctx, x, W, bias, mask, relu, True)
        want = conv_ref(x, W, bias, mask, relu)
        assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()


def test_conv_bf16_out_and_channel_slice(ctx):
    x, W, bias, mask = case((13, 11, 17), 32, 32, 5)
    got = run_conv(ctx, x, W, bias, mask, 1, False)
    want = conv_ref(x, W, bias, mask, 1)
    assert np.all(np.abs(got - want) <= 2.0 ** -8 * np.abs(want) + 1e-6)
    # only the first channel, FP32 (the preconditioner's output layer)
    got1 = run_conv(ctx, x, W, None, mask, 0, True, out_ch=1)
    want1 = conv_ref(x, W, None, mask, 0)[..., :1]
    assert np.abs(got1 - want1).max() <= 1e-5 * np.abs(want1).max()
