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
