"""Test infrastructure only: numpy FP64 restatement of the learned
preconditioner (the 3-level 3-D U-Net of xflow_gb300/csrc/xf_unet.cu) with
its loss and backward pass, the checker of the GPU's forward and gradients.

The reference has no learned component; this restatement follows the
network as the library defines it (levels, masks, pooling, upsampling,
channel slices, loss) and is exact FP64 arithmetic (the GPU keeps BF16
weights and activations, so comparisons carry BF16-level tolerances).
"""
import numpy as np

LAYERS = (("enc0a", 16, 16), ("enc0b", 16, 16), ("enc1a", 16, 32), ("enc1b", 32, 32), ("mid_a", 32, 64),
          ("mid_b", 64, 64), ("dec1a", 96, 32), ("dec1b", 32, 32), ("dec0a", 48, 16), ("dec0b", 16, 16),
          ("out", 16, 16))


def unpack(p):
    out, o = {}, 0
    for name, ci, co in LAYERS:
        w = p[o:o + 27 * co * ci].reshape(27, co, ci).astype(np.float64)
        o += 27 * co * ci
        b = p[o:o + co].astype(np.float64)
        o += co
        out[name] = (w, b)
    return out


def pack(d):
    return np.concatenate([np.concatenate([d[n][0].ravel(), d[n][1].ravel()]) for n, _, _ in LAYERS])


def coarse_mask(m):
    n1, n2, n3 = m.shape
    c = np.zeros(((n1 - 2) // 2 + 2, (n2 - 2) // 2 + 2, (n3 - 2) // 2 + 2))
    inner = m[1:-1, 1:-1, 1:-1].reshape((n1 - 2) // 2, 2, (n2 - 2) // 2, 2, (n3 - 2) // 2, 2)
    c[1:-1, 1:-1, 1:-1] = inner.max(axis=(1, 3, 5))
    return (c > 0).astype(np.float64)


def _shift(x, di, dj, dk):
    """y[i,j,k] = x[i+di, j+dj, k+dk], 0 outside the box."""
    y = np.zeros_like(x)
    n1, n2, n3 = x.shape[:3]
    sl = lambda d, n: (slice(max(0, -d), n - max(0, d)), slice(max(0, d), n - max(0, -d)))  # noqa: E731
    (a0, a1), (b0, b1), (c0, c1) = sl(di, n1), sl(dj, n2), sl(dk, n3)
    y[a0, b0, c0] = x[a1, b1, c1]
    return y


def conv(x, w, b=None):
    """x [n1,n2,n3,ci], w [27,co,ci] -> [n1,n2,n3,co] (+ b)."""
    y = 0.0
    for t in range(27):
        y = y + _shift(x, t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) @ w[t].T
    return y + (b if b is not None else 0.0)


def conv_wgrad(g, x):
    """d/dw of sum(g * conv(x, w)): [27, co, ci]."""
    co, ci = g.shape[-1], x.shape[-1]
    gw = np.zeros((27, co, ci))
    for t in range(27):
        xs = _shift(x, t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1)
        gw[t] = g.reshape(-1, co).T @ xs.reshape(-1, ci)
    return gw


def conv_dgrad(g, w):
    """d/dx of sum(g * conv(x, w)): conv of g with the flipped transposed weights."""
    wt = np.stack([w[26 - t].T for t in range(27)])
    return conv(g, wt)


def pool(x, mc):
    n1, n2, n3, C = x.shape
    y = np.zeros(mc.shape + (C,))
    inner = x[1:-1, 1:-1, 1:-1].reshape((n1 - 2) // 2, 2, (n2 - 2) // 2, 2, (n3 - 2) // 2, 2, C)
    y[1:-1, 1:-1, 1:-1] = inner.mean(axis=(1, 3, 5))
    return y * mc[..., None]


def pool_bwd(g, mf):
    return upsample(g, mf) / 8.0


def upsample(x, mf):
    y = np.zeros(mf.shape + (x.shape[-1],))
    inner = x[1:-1, 1:-1, 1:-1]
    y[1:-1, 1:-1, 1:-1] = inner.repeat(2, 0).repeat(2, 1).repeat(2, 2)
    return y * mf[..., None]


def upsample_bwd(g, mc):
    n1, n2, n3, C = g.shape
    y = np.zeros(mc.shape + (C,))
    inner = g[1:-1, 1:-1, 1:-1].reshape((n1 - 2) // 2, 2, (n2 - 2) // 2, 2, (n3 - 2) // 2, 2, C)
    y[1:-1, 1:-1, 1:-1] = inner.sum(axis=(1, 3, 5))
    return y * mc[..., None]


def forward(params, r, m0):
    P = unpack(params)
    m1 = coarse_mask(m0)
    m2 = coarse_mask(m1)
    M = {0: m0[..., None], 1: m1[..., None], 2: m2[..., None]}
    act = {}
    rms = np.sqrt((r[m0 > 0] ** 2).mean())
    x0 = np.zeros(r.shape + (16,))
    x0[..., 0] = r / rms * m0
    act["x0"] = x0

    def layer(name, x, lev, relu=True):
        y = conv(x, *P[name])
        if relu:
            y = np.maximum(y, 0)
        return y * M[lev]

    act["a0"] = layer("enc0a", x0, 0)
    act["s0"] = layer("enc0b", act["a0"], 0)
    act["p1"] = pool(act["s0"], m1)
    act["a1"] = layer("enc1a", act["p1"], 1)
    act["s1"] = layer("enc1b", act["a1"], 1)
    act["p2"] = pool(act["s1"], m2)
    act["m2a"] = layer("mid_a", act["p2"], 2)
    act["m2b"] = layer("mid_b", act["m2a"], 2)
    act["cat1"] = np.concatenate([upsample(act["m2b"], m1), act["s1"]], -1)
    act["d1a"] = layer("dec1a", act["cat1"], 1)
    act["d1b"] = layer("dec1b", act["d1a"], 1)
    act["cat0"] = np.concatenate([upsample(act["d1b"], m0), act["s0"]], -1)
    act["d0a"] = layer("dec0a", act["cat0"], 0)
    act["d0b"] = layer("dec0b", act["d0a"], 0)
    z = layer("out", act["d0b"], 0, relu=False)[..., 0]
    return z, (P, M, m0, m1, m2, act)


def loss_and_grads(params, r, e, m0, apply_A=None):
    """Loss and its parameter gradient.  Without apply_A: mean over active
    cells of (z - e / rms e)^2.  With apply_A (the symmetric operator, A e = r):
    one minus the A-norm cosine (z, r) / sqrt((z, A z) (e, r)) between the
    output and the error, the quantity preconditioned CG convergence depends
    on (signed, so that the output is a descent direction)."""
    z, (P, M, m0, m1, m2, a) = forward(params, r, m0)
    act0 = m0 > 0
    cnt = act0.sum()
    gz = np.zeros(z.shape + (16,))
    if apply_A is None:
        t = e / np.sqrt((e[act0] ** 2).mean())
        d = (z - t) * m0
        loss = (d[act0] ** 2).sum() / cnt
        gz[..., 0] = 2 * d / cnt
    else:
        zm = z * m0
        az = apply_A(zm) * m0
        zr, zaz, er = (zm * r).sum(), (zm * az).sum(), (e * r * m0).sum()
        loss = 1 - zr / np.sqrt(zaz * er)
        gz[..., 0] = -(r - zr / zaz * az) / np.sqrt(zaz * er) * m0
    G = {}

    def back(name, g, x, gate=None, lev=0):
        """g: pre-activation gradient of `name`; returns dL/dx (before x's own gate)."""
        G[name] = (conv_wgrad(g, x), g.reshape(-1, g.shape[-1]).sum(0))
        return conv_dgrad(g, P[name][0]) * M[lev]

    relu_g = lambda g, y: g * (y > 0)  # noqa: E731
    g = back("out", gz, a["d0b"], lev=0)
    g = back("dec0b", relu_g(g, a["d0b"]), a["d0a"], lev=0)
    g = back("dec0a", relu_g(g, a["d0a"]), a["cat0"], lev=0)
    g_up0, g_s0 = g[..., :32], g[..., 32:]
    g = upsample_bwd(g_up0, m1)
    g = back("dec1b", relu_g(g, a["d1b"]), a["d1a"], lev=1)
    g = back("dec1a", relu_g(g, a["d1a"]), a["cat1"], lev=1)
    g_up1, g_s1 = g[..., :64], g[..., 64:]
    g = upsample_bwd(g_up1, m2)
    g = back("mid_b", relu_g(g, a["m2b"]), a["m2a"], lev=2)
    g = back("mid_a", relu_g(g, a["m2a"]), a["p2"], lev=2)
    g_s1 = g_s1 + pool_bwd(g, m1)
    g = back("enc1b", relu_g(g_s1, a["s1"]) * M[1], a["a1"], lev=1)
    g = back("enc1a", relu_g(g, a["a1"]), a["p1"], lev=1)
    g_s0 = g_s0 + pool_bwd(g, m0)
    g = back("enc0b", relu_g(g_s0, a["s0"]) * M[0], a["a0"], lev=0)
    back("enc0a", relu_g(g, a["a0"]), a["x0"], lev=0)
    return loss, pack(G), z
