"""Test infrastructure only: ctypes front of oracle/liboracle.so, the CPU
restatement of the reference arithmetic (oracle/xf_oracle.c).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the
checker.  The product never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

LAPLACE, VARDIV = 0, 1


XFO_OK, XFO_ERR_ARG, XFO_ERR_MASK, XFO_ERR_CHECK = 0, 1, 3, 7   # oracle status codes (xf_oracle.h)

def build():
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        d, i32, i64, u8 = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_uint8)
        L.xfo_rn_map.restype = C.c_int64
        L.xfo_dot.restype = C.c_double
        L.xfo_norm.restype = C.c_double
        L.xfo_absmax.restype = C.c_double
        L.xfo_divergence_max.restype = C.c_double
        L.xfo_pack_build.restype = C.c_int64
        L.xfo_format_fixed6.restype = C.c_int64
        L.xfo_format_fixed6.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64]
        L.xfo_pack_apply.argtypes = [C.c_int64] + [C.c_void_p] * 5
        L.xfo_bicg_reference.argtypes = [C.c_int64] + [C.c_void_p] * 7 + [C.c_double, C.c_int, C.c_void_p,
                                                                          C.c_void_p]
        _lib = L
    return _lib


class Stats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("resid", C.c_double), ("status", C.c_int)]


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def set_threads(n):
    lib().xfo_set_threads(int(n))


def space_mask(codes):
    codes = np.ascontiguousarray(codes, dtype=np.int32)
    out = np.empty(codes.shape, np.uint8)
    lib().xfo_space_mask(_p(codes, C.c_int32), C.c_int64(codes.size), _p(out, C.c_uint8))
    return out


def rn_map(smask):
    smask = np.ascontiguousarray(smask, dtype=np.uint8)
    n1, n2, n3 = smask.shape
    inv = np.zeros(smask.shape, np.int32)
    cnt = int(smask.sum())
    fwd = np.zeros((cnt, 3), np.int32)
    r = lib().xfo_rn_map(_p(smask, C.c_uint8), n1, n2, n3, _p(inv, C.c_int32), _p(fwd, C.c_int32))
    return int(r), inv, fwd


def validate(op, codes, normals):
    codes = np.ascontiguousarray(codes, dtype=np.int32)
    normals = f64(normals)
    bad = C.c_int64(-1)
    st = lib().xfo_validate(op, _p(codes, C.c_int32), _p(normals, C.c_double), *codes.shape, C.byref(bad))
    return st, bad.value


class Grid:
    """Codes, normals, separations (and density) of one box."""

    def __init__(self, codes, normals, hx, hy, hz, density=None):
        self.codes = np.ascontiguousarray(codes, dtype=np.int32)
        self.normals = f64(normals)
        self.hx, self.hy, self.hz = f64(hx), f64(hy), f64(hz)
        self.density = f64(density) if density is not None else np.ones(self.codes.shape)
        self.shape = self.codes.shape
        self.smask = space_mask(self.codes)

    def args(self):
        return (_p(self.codes, C.c_int32), _p(self.normals, C.c_double), _p(self.hx, C.c_double),
                _p(self.hy, C.c_double), _p(self.hz, C.c_double), _p(self.density, C.c_double), *self.shape)


def apply(op, g, x, s=None, sign=0, y_init=None):
    x = f64(x)
    y = f64(y_init).copy() if y_init is not None else np.zeros(g.shape)
    s_ = f64(s) if s is not None else np.zeros(g.shape)
    st = lib().xfo_apply(op, *g.args(), _p(x, C.c_double), _p(s_, C.c_double), sign, _p(y, C.c_double))
    if st != 0:
        raise ValueError(f"oracle apply rejected the grid (status {st})")
    return y


def lincomb(p1, s1, p2, s2, smask, z_init):
    z = f64(z_init).copy()
    s1 = f64(s1)
    s2k = f64(s2) if s2 is not None else None
    lib().xfo_lincomb(C.c_double(p1), _p(s1, C.c_double), C.c_double(p2),
                      _p(s2k, C.c_double) if s2k is not None else None,
                      _p(np.ascontiguousarray(smask, np.uint8), C.c_uint8), C.c_int64(z.size), _p(z, C.c_double))
    return z


def dot(a, b, smask):
    a, b = f64(a), f64(b)
    m = np.ascontiguousarray(smask, np.uint8)
    return lib().xfo_dot(_p(a, C.c_double), _p(b, C.c_double), _p(m, C.c_uint8), C.c_int64(a.size))


def norm(a, smask):
    a = f64(a)
    m = np.ascontiguousarray(smask, np.uint8)
    return lib().xfo_norm(_p(a, C.c_double), _p(m, C.c_uint8), C.c_int64(a.size))


def absmax(a, smask, inv):
    a = f64(a)
    m = np.ascontiguousarray(smask, np.uint8)
    inv = np.ascontiguousarray(inv, np.int32)
    idx = C.c_int32(0)
    v = lib().xfo_absmax(_p(a, C.c_double), _p(m, C.c_uint8), _p(inv, C.c_int32), C.c_int64(a.size), C.byref(idx))
    return v, idx.value


def _solve(fn, op, g, x0, b, tol, maxit):
    x0, b = f64(x0), f64(b)
    res = np.zeros(g.shape)
    st = Stats()
    rc = fn(op, *g.args(), _p(x0, C.c_double), _p(b, C.c_double), C.c_double(tol), int(maxit),
            _p(res, C.c_double), C.byref(st))
    if rc != 0:
        raise ValueError(f"oracle solver rejected the grid (status {rc})")
    return res, st


def cg_reference(op, g, x0, b, eps=0.0, maxit=0):
    return _solve(lib().xfo_cg_reference, op, g, x0, b, eps, maxit)


def bicgstab_reference(op, g, x0, b, eps=0.0, maxit=0):
    return _solve(lib().xfo_bicgstab_reference, op, g, x0, b, eps, maxit)


def minres_reference(op, g, x0, b, eps=0.0, maxit=0):
    return _solve(lib().xfo_minres_reference, op, g, x0, b, eps, maxit)


def cg_plain(op, g, x0, b, rtol, maxit=0):
    return _solve(lib().xfo_cg_plain, op, g, x0, b, rtol, maxit)


def thomas(M, u, a, b, c, f):
    u = f64(u).copy()
    lib().xfo_thomas(int(M), _p(u, C.c_double), _p(f64(a), C.c_double), _p(f64(b), C.c_double),
                     _p(f64(c), C.c_double), _p(f64(f), C.c_double))
    return u


def ib_interpolate(vel, h0, axis, pos):
    vel, h0, pos = f64(vel), f64(h0), f64(pos)
    out = np.zeros(len(pos))
    lib().xfo_ib_interpolate(_p(vel, C.c_double), *vel.shape, _p(h0, C.c_double), int(axis), len(pos),
                             _p(pos, C.c_double), _p(out, C.c_double))
    return out


def ib_update(axis, tau, node_vel, pos):
    pos = f64(pos).copy()
    lib().xfo_ib_update(len(pos), int(axis), C.c_double(tau), _p(f64(node_vel), C.c_double), _p(pos, C.c_double))
    return pos


def ib_forces(axis, pos, ref, kind, nxt, prv, dist0, curv0, node_stiff, params):
    n = len(kind)
    out = np.zeros(n)
    i32 = lambda a: np.ascontiguousarray(a, np.int32)  # noqa: E731
    kind, nxt, prv = i32(kind), i32(nxt), i32(prv)
    lib().xfo_ib_forces(n, int(axis), _p(f64(pos), C.c_double), _p(f64(ref), C.c_double), _p(kind, C.c_int32),
                        _p(nxt, C.c_int32), _p(prv, C.c_int32), _p(f64(dist0), C.c_double),
                        _p(f64(curv0), C.c_double), _p(f64(node_stiff), C.c_double), _p(f64(params), C.c_double),
                        _p(out, C.c_double))
    return out


def ib_spread(shape, h0, axis, pos, force, fbox=None):
    fbox = np.zeros(shape) if fbox is None else f64(fbox).copy()
    pos, h0 = f64(pos), f64(h0)
    lib().xfo_ib_spread(_p(fbox, C.c_double), *shape, _p(h0, C.c_double), int(axis), len(pos),
                        _p(pos, C.c_double), _p(f64(force), C.c_double))
    return fbox


# Time-step passes (XProblem.cpp:5474-5829)
def pressure_rhs(codes, u, v, w, hxU, hyV, hzW, tau, density=None, border=None):
    codes = np.ascontiguousarray(codes, np.int32)
    rhs = np.zeros(codes.shape)
    bad = C.c_int64(-1)
    st = lib().xfo_pressure_rhs(_p(codes, C.c_int32), *codes.shape, _p(f64(u), C.c_double), _p(f64(v), C.c_double),
                                _p(f64(w), C.c_double), _p(f64(hxU), C.c_double), _p(f64(hyV), C.c_double),
                                _p(f64(hzW), C.c_double), _p(f64(density), C.c_double) if density is not None else None,
                                C.c_double(tau), _p(f64(border), C.c_double) if border is not None else None,
                                _p(rhs, C.c_double), C.byref(bad))
    return rhs, st, bad.value


def velocity_correct(axis, codes, prev, p, hP, tau, density=None, border=None, cur=None):
    codes = np.ascontiguousarray(codes, np.int32)
    cur = np.zeros(codes.shape) if cur is None else f64(cur).copy()
    bad = C.c_int64(-1)
    st = lib().xfo_velocity_correct(int(axis), _p(codes, C.c_int32), *codes.shape, _p(f64(prev), C.c_double),
                                    _p(f64(p), C.c_double), _p(f64(hP), C.c_double),
                                    _p(f64(density), C.c_double) if density is not None else None, C.c_double(tau),
                                    _p(f64(border), C.c_double) if border is not None else None,
                                    _p(cur, C.c_double), C.byref(bad))
    return cur, st, bad.value


def momentum_rhs(axis, codes, u, v, w, hx, hy, hz, vis=None, border=None, force=None, normals=None):
    """Momentum right-hand side of velocity component `axis` on its own box (XProblem.cpp:5088-5419):
    returns (uTr, vTr, wTr, visTr, rp), status, first throwing cell."""
    codes = np.ascontiguousarray(codes, np.int32)
    out = [np.zeros(codes.shape) for _ in range(5)]
    bad = C.c_int64(-1)
    p = lambda a: _p(f64(a), C.c_double) if a is not None else None  # noqa: E731
    st = lib().xfo_momentum_rhs(int(axis), _p(codes, C.c_int32), p(normals), *codes.shape, p(u), p(v), p(w), p(vis),
                                p(hx), p(hy), p(hz), p(border), p(force), *(_p(o, C.c_double) for o in out),
                                C.byref(bad))
    return tuple(out), st, bad.value


def adi_line_coeffs(direction, codes, hx, hy, hz, vec_tr, D, tau):
    """The reference's ADI line coefficients (a, b, c) along `direction` at every Actual point
    (XProblem.cpp:3149-3190); NaN elsewhere."""
    codes = np.ascontiguousarray(codes, np.int32)
    out = [np.full(codes.shape, np.nan) for _ in range(3)]
    lib().xfo_adi_line_coeffs(int(direction), _p(codes, C.c_int32), *codes.shape, _p(f64(hx), C.c_double),
                              _p(f64(hy), C.c_double), _p(f64(hz), C.c_double), _p(f64(vec_tr), C.c_double),
                              _p(f64(D), C.c_double), C.c_double(tau), *(_p(o, C.c_double) for o in out))
    return tuple(out)


def adi_first_rhs(codes, hx, hy, hz, f_1, u, v, w, D, rp, tau):
    """The right-hand side of the first splitting step's x lines at every Actual point
    (XProblem.cpp:3192-3276); NaN elsewhere."""
    codes = np.ascontiguousarray(codes, np.int32)
    f = np.full(codes.shape, np.nan)
    d = lambda a: _p(f64(a), C.c_double)  # noqa: E731
    lib().xfo_adi_first_rhs(_p(codes, C.c_int32), *codes.shape, d(hx), d(hy), d(hz), d(f_1), d(u), d(v), d(w), d(D),
                            d(rp), C.c_double(tau), _p(f, C.c_double))
    return f


def adi_upwind_coeffs(direction, codes, hx, hy, hz, vec_tr, D, tau):
    """The concentration's upwind ADI line coefficients (a, b, c) along `direction` at every Actual
    point (SolveTransferEquation_, schemeType 1, XProblem.cpp:1828-1843); NaN elsewhere."""
    codes = np.ascontiguousarray(codes, np.int32)
    out = [np.full(codes.shape, np.nan) for _ in range(3)]
    lib().xfo_adi_upwind_coeffs(int(direction), _p(codes, C.c_int32), *codes.shape, _p(f64(hx), C.c_double),
                                _p(f64(hy), C.c_double), _p(f64(hz), C.c_double), _p(f64(vec_tr), C.c_double),
                                C.c_double(D), C.c_double(tau), *(_p(o, C.c_double) for o in out))
    return tuple(out)


def adi_first_rhs_upwind(codes, hx, hy, hz, f_1, u, v, w, D, rp, tau):
    """The upwind first-direction right-hand side at every Actual point (XProblem.cpp:1848-1912 with
    schemeType 1) for a scalar diffusion coefficient D; NaN elsewhere."""
    codes = np.ascontiguousarray(codes, np.int32)
    out = np.full(codes.shape, np.nan)
    d = lambda a: _p(f64(a), C.c_double)  # noqa: E731
    lib().xfo_adi_first_rhs_upwind(_p(codes, C.c_int32), *codes.shape, d(hx), d(hy), d(hz), d(f_1), d(u), d(v),
                                   d(w), C.c_double(D), d(rp), C.c_double(tau), _p(out, C.c_double))
    return out


def conc_transfer(codes, u, v, w, inlet=None):
    """The concentration equation's transfer terms (uTr, vTr, wTr, rpTr) on its grid
    (XProblem.cpp:5886-5935); status 1 (a point type the reference throws on) or 2 (an Actual point on the
    box face) and the flat index of the first such point."""
    codes = np.ascontiguousarray(codes, np.int32)
    out = [np.zeros(codes.shape) for _ in range(4)]
    bad = C.c_int64(-1)
    st = lib().xfo_conc_transfer(_p(codes, C.c_int32), *codes.shape, _p(f64(u), C.c_double), _p(f64(v), C.c_double),
                                 _p(f64(w), C.c_double), _p(f64(inlet), C.c_double) if inlet is not None else None,
                                 *(_p(o, C.c_double) for o in out), C.byref(bad))
    return tuple(out), st, bad.value


def divergence_max(codes, u, v, w, hxU, hyV, hzW):
    codes = np.ascontiguousarray(codes, np.int32)
    ijk = np.zeros(3, np.int32)
    val = lib().xfo_divergence_max(_p(codes, C.c_int32), *codes.shape, _p(f64(u), C.c_double),
                                   _p(f64(v), C.c_double), _p(f64(w), C.c_double), _p(f64(hxU), C.c_double),
                                   _p(f64(hyV), C.c_double), _p(f64(hzW), C.c_double), _p(ijk, C.c_int32))
    return val, tuple(int(t) for t in ijk)


# T1dPackOperator and the reference BiCG (XOperator.cpp:1135-1571, XSLAE.cpp:159-348)
class Pack:
    def __init__(self, a_ptr, a_cols, a_vals, t_ptr, t_cols, t_vals):
        self.a = (np.ascontiguousarray(a_ptr, np.int32), np.ascontiguousarray(a_cols, np.int32), f64(a_vals))
        self.t = (np.ascontiguousarray(t_ptr, np.int32), np.ascontiguousarray(t_cols, np.int32), f64(t_vals))
        self.rows = len(self.a[0]) - 1


def pack_build(op, g):
    R = int(g.smask.sum())
    a_ptr, t_ptr = np.zeros(R + 1, np.int32), np.zeros(R + 1, np.int32)
    a_cols, t_cols = np.zeros(7 * R, np.int32), np.zeros(7 * R, np.int32)
    a_vals, t_vals = np.zeros(7 * R), np.zeros(7 * R)
    nnz = lib().xfo_pack_build(op, *g.args(), _p(a_ptr, C.c_int32), _p(a_cols, C.c_int32),
                               _p(a_vals, C.c_double), _p(t_ptr, C.c_int32), _p(t_cols, C.c_int32),
                               _p(t_vals, C.c_double))
    if nnz < 0:
        raise ValueError("the operator rejects this grid")
    return Pack(a_ptr, a_cols[:nnz], a_vals[:nnz], t_ptr, t_cols[:nnz], t_vals[:nnz])


def pack_apply(pk, x, transpose=False):
    ptr, cols, vals = pk.t if transpose else pk.a
    y = np.zeros(pk.rows)
    lib().xfo_pack_apply(pk.rows, _p(ptr, C.c_int32), _p(cols, C.c_int32), _p(vals, C.c_double),
                         _p(f64(x), C.c_double), _p(y, C.c_double))
    return y


def bicg_reference(pk, b, eps=0.0, maxit=0):
    out = np.zeros(pk.rows)
    st = Stats()
    rc = lib().xfo_bicg_reference(pk.rows, *[_p(a, C.c_int32 if a.dtype == np.int32 else C.c_double)
                                             for a in pk.a + pk.t],
                                  _p(f64(b), C.c_double), C.c_double(eps), int(maxit), _p(out, C.c_double),
                                  C.byref(st))
    return out, st, rc


def apply_advdiff(g, x, u, v, w, tau, D, flags=3, Dfield=None):
    """Implicit advection-diffusion operator on the oracle grid g (XProblem.cpp:1236-1238 summed over x, y, z);
    Dfield: the per-cell diffusion coefficient of the variable-viscosity form (XProblem.cpp:3204)."""
    y = np.zeros(g.shape)
    p = lambda a: _p(f64(a), C.c_double) if a is not None else None  # noqa: E731
    st = lib().xfo_apply_advdiff(_p(g.codes, C.c_int32), _p(g.normals, C.c_double), _p(g.hx, C.c_double),
                                 _p(g.hy, C.c_double), _p(g.hz, C.c_double), p(u), p(v), p(w), C.c_double(tau),
                                 C.c_double(D), p(Dfield), int(flags), *g.shape, _p(f64(x), C.c_double),
                                 _p(y, C.c_double))
    if st != 0:
        raise ValueError("oracle advection-diffusion rejected the grid")
    return y


# Field output (XProblem.cpp:6132-6345)
def vtk_write(path, node_codes, x, y, z, u, v, w, p_codes, p, d_codes, density, c_codes, conc, vis):
    """The reference's VTK legacy ASCII volume written with its own format strings; node box shape (N+1, L+1, M+1)."""
    N, L, M = (s_ - 1 for s_ in node_codes.shape)
    i32 = lambda a: _p(np.ascontiguousarray(a, np.int32), C.c_int32)  # noqa: E731
    d = lambda a: _p(f64(a), C.c_double)  # noqa: E731
    keep = [np.ascontiguousarray(a, np.int32) for a in (node_codes, p_codes, d_codes, c_codes)]
    st = lib().xfo_vtk_write(str(path).encode(), N, L, M, i32(keep[0]), d(x), d(y), d(z), d(u), d(v), d(w),
                             i32(keep[1]), d(p), i32(keep[2]), d(density), i32(keep[3]), d(conc), d(vis))
    if st != 0:
        raise OSError("oracle VTK writer could not open " + str(path))


def format_fixed6(values):
    """b"".join(b"%f\n" % v): the C library's "%f" of each value."""
    v = f64(values)
    n = lib().xfo_format_fixed6(_p(v, C.c_double), v.size, None, 0)
    buf = C.create_string_buffer(int(n))
    lib().xfo_format_fixed6(_p(v, C.c_double), v.size, buf, n)
    return buf.raw[:n]


def voxelize_mesh(codes, x_nodes, y_nodes, z_nodes, vertices, faces, inside_code):
    """Checker of the library's voxeliser (no counterpart in the reference,
    which uses STL vertices only as markers, XImmersedBoundary.cpp:1560-1570;
    parity unpinned by the reference).  The same rule, restated with numpy:
    rays along x at (y[j], z[k]); a triangle is crossed where the ray's (y, z)
    lies in its (y, z) projection, points on a projected edge counted by the
    top-left rule of the counter-clockwise traversal; edge functions from the
    endpoints in lexicographic order, negated for the other direction; a point
    is inside when an odd number of crossing abscissae lie below its x.  Every
    product and sum is rounded on its own, as on the device."""
    out = np.array(codes, dtype=np.int32, copy=True)
    x_nodes, y_nodes, z_nodes = (np.asarray(a, dtype=np.float64) for a in (x_nodes, y_nodes, z_nodes))
    V = np.asarray(vertices, dtype=np.float64).reshape(-1, 3)
    F = np.asarray(faces, dtype=np.int64).reshape(-1, 3)
    A, B, C = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]

    def edge_fn(a, b, pu, pv):
        """a, b: (m, 2) endpoints (u = y, v = z); pu, pv: (r, 1) points -> (r, m)."""
        fwd = (a[:, 0] < b[:, 0]) | ((a[:, 0] == b[:, 0]) & (a[:, 1] < b[:, 1]))
        s = np.where(fwd[:, None], a, b)
        t = np.where(fwd[:, None], b, a)
        du, dv = t[:, 0] - s[:, 0], t[:, 1] - s[:, 1]
        e = du * (pv - s[:, 1]) - dv * (pu - s[:, 0])
        return np.where(fwd, e, -e)

    def top_left(a, b):
        du, dv = b[:, 0] - a[:, 0], b[:, 1] - a[:, 1]
        return (dv < 0.0) | ((dv == 0.0) & (du > 0.0))

    a2, b2_, c2_ = A[:, 1:], B[:, 1:], C[:, 1:]
    # area of each projected triangle: the edge function of a -> b at c
    fwd = (a2[:, 0] < b2_[:, 0]) | ((a2[:, 0] == b2_[:, 0]) & (a2[:, 1] < b2_[:, 1]))
    s = np.where(fwd[:, None], a2, b2_)
    t = np.where(fwd[:, None], b2_, a2)
    ar = (t[:, 0] - s[:, 0]) * (c2_[:, 1] - s[:, 1]) - (t[:, 1] - s[:, 1]) * (c2_[:, 0] - s[:, 0])
    area = np.where(fwd, ar, -ar)
    keep = area != 0.0
    ccw = area > 0
    bb = np.where(ccw[:, None], b2_, c2_)[keep]
    cc = np.where(ccw[:, None], c2_, b2_)[keep]
    aa = a2[keep]
    xa = A[keep, 0]
    xb = np.where(ccw, B[:, 0], C[:, 0])[keep]
    xc = np.where(ccw, C[:, 0], B[:, 0])[keep]
    tl0, tl1, tl2 = top_left(aa, bb), top_left(bb, cc), top_left(cc, aa)
    n1, n2, n3 = out.shape
    jj, kk = np.meshgrid(np.arange(n2), np.arange(n3), indexing="ij")
    jj, kk = jj.ravel(), kk.ravel()
    for r0 in range(0, jj.size, 256):
        j, k = jj[r0:r0 + 256], kk[r0:r0 + 256]
        pu, pv = y_nodes[j][:, None], z_nodes[k][:, None]
        e0, e1, e2 = edge_fn(aa, bb, pu, pv), edge_fn(bb, cc, pu, pv), edge_fn(cc, aa, pu, pv)
        inside = (((e0 > 0) | ((e0 == 0) & tl0)) & ((e1 > 0) | ((e1 == 0) & tl1)) &
                  ((e2 > 0) | ((e2 == 0) & tl2)))
        with np.errstate(invalid="ignore", divide="ignore"):
            x = ((e1 * xa + e2 * xb) + e0 * xc) / ((e1 + e2) + e0)
        for q in range(j.size):
            xs = np.sort(x[q][inside[q]])
            if xs.size == 0:
                continue
            below = np.searchsorted(xs, x_nodes, side="left")   # crossings strictly below each x[i]
            sel = (below & 1) == 1
            out[sel, j[q], k[q]] = inside_code
    return out
