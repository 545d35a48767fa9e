"""xf_dot_noalloc, the inner product for callers that cannot allocate device
memory (an application pooling all of its device memory at start-up under a
fixed budget, or a loop that must not call cudaFree and so wait for the whole
device to go idle): it must agree
with xf_dot, the allocating entry point, call after call, while keeping its
scratch in a static device array.

Collected last (file name) so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import xflow_gb300 as xf
from xflow_gb300 import capi
from xflow_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def test_dot_noalloc_matches_xf_dot_twice_in_a_row():
    torch = pytest.importorskip("torch")
    ctx = xf.Context(0)
    try:
        codes, nrm = wl.mixed_grid(23, 19, 26, seed=77)
        rng = np.random.Generator(np.random.PCG64(78))
        sep = [rng.uniform(0.5, 1.5, n - 1) for n in codes.shape]
        g = xf.Grid(ctx, codes, *sep, nrm)
        a_host = rng.standard_normal(g.shape)
        b_host = rng.standard_normal(g.shape)
        va, vb = g.vec(a_host), g.vec(b_host)
        want = va.dot(vb)                          # the allocating entry point
        mask = torch.from_numpy(g.space_mask().ravel().copy()).to("cuda")
        out = torch.full((1,), np.nan, dtype=torch.float64, device="cuda")
        n = int(np.prod(g.shape))
        L = capi.lib()
        stream = L.xf_stream(ctx.h)
        for _ in range(2):                         # the shared scratch must start clean each time
            out.fill_(np.nan)
            torch.cuda.synchronize()
            st = L.xf_dot_noalloc(L.xf_vec_data(va.h), L.xf_vec_data(vb.h), C.c_void_p(mask.data_ptr()),
                                  C.c_int64(n), C.c_void_p(out.data_ptr()), stream)
            assert st == capi.XF_OK
            ctx.synchronize()
            got = float(out.item())
            assert got == pytest.approx(want, rel=1e-13, abs=1e-13)
        # without a mask: every element
        st = L.xf_dot_noalloc(L.xf_vec_data(va.h), L.xf_vec_data(vb.h), None, C.c_int64(n),
                              C.c_void_p(out.data_ptr()), stream)
        assert st == capi.XF_OK
        ctx.synchronize()
        assert float(out.item()) == pytest.approx(float(np.dot(a_host.ravel(), b_host.ravel())), rel=1e-12)
        # sizes beyond the static scratch are refused
        st = L.xf_dot_noalloc(L.xf_vec_data(va.h), L.xf_vec_data(vb.h), None, C.c_int64(8192 * 256 * 16 + 1),
                              C.c_void_p(out.data_ptr()), stream)
        assert st == capi.XF_ERR_ARG
    finally:
        ctx.close()


@pytest.mark.parametrize("n", [3_000_001, 8192 * 256 * 16])
def test_dot_noalloc_many_blocks_and_the_maximum_size(n):
    """Hundreds to thousands of blocks (the last block's loop over the partials
    runs several rounds), masked and unmasked, up to exactly the largest
    accepted size; checked against an order-independent bound
    |got - exact| <= 1e-13 sum |a b|."""
    torch = pytest.importorskip("torch")
    import math

    ctx = xf.Context(0)
    try:
        gen = torch.Generator(device="cpu").manual_seed(n % 1000)
        a_h = torch.randn(n, dtype=torch.float64, generator=gen)
        b_h = torch.randn(n, dtype=torch.float64, generator=gen)
        m_h = (torch.rand(n, generator=gen) < 0.7).to(torch.uint8)
        a, b, m = a_h.cuda(), b_h.cuda(), m_h.cuda()
        out = torch.full((1,), np.nan, dtype=torch.float64, device="cuda")
        L = capi.lib()
        stream = L.xf_stream(ctx.h)
        prod = (a_h * b_h).numpy()
        for mask in (m, None):
            terms = prod[m_h.numpy().astype(bool)] if mask is not None else prod
            exact = math.fsum(terms)
            for _ in range(2):
                out.fill_(np.nan)
                torch.cuda.synchronize()
                st = L.xf_dot_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                                      C.c_void_p(mask.data_ptr()) if mask is not None else None, C.c_int64(n),
                                      C.c_void_p(out.data_ptr()), stream)
                assert st == capi.XF_OK
                ctx.synchronize()
                assert abs(float(out.item()) - exact) <= 1e-13 * float(np.abs(terms).sum())
    finally:
        ctx.close()

