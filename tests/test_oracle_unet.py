"""The numpy restatement of the U-Net (oracle/unet_ref.py), the checker of the
GPU's gradients, checked on its own: its analytic gradient against central
finite differences of its loss (FP64, 1e-5 relative)."""
import numpy as np

from oracle import unet_ref as U
from xflow_gb300 import workloads as wl


import pytest


@pytest.mark.parametrize("anorm", [False, True])
def test_oracle_gradient_matches_finite_differences(anorm):
    codes, _, _, _, _ = wl.spheres_grid(8, 1, 0.15, 0.2, 3)
    m0 = wl.space_mask(codes).astype(np.float64)
    rng = np.random.Generator(np.random.PCG64(11))
    r = rng.standard_normal(codes.shape) * m0
    e = rng.standard_normal(codes.shape) * m0
    apply_A = None
    if anorm:
        from oracle import oracle as O

        og = O.Grid(codes, np.zeros(codes.shape + (3,)), *(np.full(n - 1, 1 / 8) for n in codes.shape))
        apply_A = lambda x: O.apply(O.LAPLACE, og, x)  # noqa: E731
        r = apply_A(e) * m0
    import xflow_gb300 as xf   # noqa: F401  (parameter layout and initialisation only)
    p = xf.unet_init_params(seed=2).astype(np.float64)
    p += rng.standard_normal(p.size) * 0.01 * (p != 0)   # leave the padding at 0
    loss, g, _ = U.loss_and_grads(p, r, e, m0, apply_A)
    idx = rng.choice(np.flatnonzero(p != 0), 12, replace=False)
    biases = []
    o = 0
    for name, ci, co in U.LAYERS:
        o += 27 * co * ci
        biases.append(o + 2)
        o += co
    for q in list(idx) + biases[2:6]:
        h = 1e-5 * max(1.0, abs(p[q]))
        pp, pm = p.copy(), p.copy()
        pp[q] += h
        pm[q] -= h
        fd = (U.loss_and_grads(pp, r, e, m0, apply_A)[0] - U.loss_and_grads(pm, r, e, m0, apply_A)[0]) / (2 * h)
        assert abs(fd - g[q]) <= 1e-5 * max(abs(fd), 1e-3 * abs(loss)), (q, fd, g[q])
