"""xflow_gb300: GB300-native pressure-projection path of xFlow.

Python front of the C ABI (include/xflow.h).  The objects mirror the
reference's surface: Grid ~ T3dNormalGrid + TRnRelease3dSpaceModel,
Vec ~ TRnRelease3dSpace, Operator ~ T3dLaplaceOperator /
T3dVariableDivergentedOperator, SLAE ~ TSLAE (XSLAE.h:9-48).  Every call runs
on the GPU through libxflow.so; a missing library raises, nothing falls back
to the CPU.
"""
import ctypes as C
import weakref

import numpy as np

from . import capi
from .capi import (XF_ADV_CONVECTIVE, XF_ADV_DIFFUSIVE, XF_ADV_UPWIND, XF_BICG, XF_BICGSTAB, XF_CG,  # noqa: F401
                   XF_CG_REFERENCE, XF_EXACT, XF_F32, XF_F64, XF_IB_FORCE, XF_IB_POS, XF_IB_VEL, XF_MINRES,
                   XF_OP_ADVDIFF, XF_OP_LAPLACE, XF_OP_VARDIV, XF_PREC_FP64, XF_PREC_MIXED, XF_PRECOND_UNET2,
                   XF_ZERO_INACTIVE, XFError)


def _check(ctx_handle, st):
    if st != capi.XF_OK:
        msg = capi.lib().xf_last_error(ctx_handle) if ctx_handle else b""
        raise XFError(st, (msg or capi.lib().xf_status_string(st)).decode())


class _Owned:
    """A handle whose children are released before it (objects may be
    collected in any order, so a child whose parent is gone is skipped)."""

    h = None

    def _init_children(self):
        self._children = weakref.WeakSet()

    def _adopt(self, child):
        self._children.add(child)

    def _close_children(self):
        for ch in list(getattr(self, "_children", ())):
            ch.close()


class Context(_Owned):
    def __init__(self, device=0):
        L = capi.lib()
        h = C.c_void_p()
        self._init_children()
        st = L.xf_create(device, C.byref(h))
        if st != capi.XF_OK:
            raise XFError(st, "xf_create failed (no CUDA device?)")
        self.h = h

    def close(self):
        if self.h:
            self._close_children()
            capi.lib().xf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self):
        _check(self.h, capi.lib().xf_synchronize(self.h))


class Grid(_Owned):
    """Box of point codes with separations and normals (reference layout)."""

    def __init__(self, ctx, codes, hx, hy, hz, normals=None):
        self.ctx = ctx
        self._init_children()
        self.codes = np.ascontiguousarray(codes, dtype=np.int32)
        self.shape = self.codes.shape
        hx, hy, hz = (np.ascontiguousarray(a, dtype=np.float64) for a in (hx, hy, hz))
        nrm = np.ascontiguousarray(normals, dtype=np.float64) if normals is not None else None
        h = C.c_void_p()
        _check(ctx.h, capi.lib().xf_grid_create(ctx.h, *self.shape, capi._ptr(self.codes), capi._ptr(hx),
                                                capi._ptr(hy), capi._ptr(hz), capi._ptr(nrm), C.byref(h)))
        self.h = h
        self._keep = (hx, hy, hz)
        ctx._adopt(self)

    @property
    def end_index(self):
        e = C.c_int64()
        _check(self.ctx.h, capi.lib().xf_grid_end_index(self.h, C.byref(e)))
        return e.value

    def rn_map(self):
        inv = np.zeros(self.shape, np.int32)
        fwd = np.zeros((self.end_index, 3), np.int32)
        _check(self.ctx.h, capi.lib().xf_grid_rn_map(self.h, capi._ptr(inv), capi._ptr(fwd)))
        return inv, fwd

    def space_mask(self):
        m = np.zeros(self.shape, np.uint8)
        _check(self.ctx.h, capi.lib().xf_grid_space_mask(self.h, capi._ptr(m)))
        return m

    def check(self, op):
        bad = C.c_int64(-1)
        st = capi.lib().xf_grid_check(self.h, op, C.byref(bad))
        return st, bad.value

    def vec(self, data=None, dtype=XF_F64):
        v = Vec(self, dtype)
        if data is not None:
            v.upload(data)
        return v

    def close(self):
        if self.h:
            self._close_children()
            if self.ctx.h:
                capi.lib().xf_grid_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Vec(_Owned):
    def __init__(self, grid, dtype=XF_F64):
        self.grid, self.dtype = grid, dtype
        h = C.c_void_p()
        _check(grid.ctx.h, capi.lib().xf_vec_create(grid.h, dtype, C.byref(h)))
        self.h = h
        grid._adopt(self)

    def upload(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.size == int(np.prod(self.grid.shape))
        _check(self.grid.ctx.h, capi.lib().xf_vec_upload(self.h, capi._ptr(a)))
        return self

    def download(self, out=None):
        """The box as a new array, or into `out` (C-contiguous float64 of the box's size, e.g. pinned memory)."""
        if out is None:
            out = np.empty(self.grid.shape, np.float64)
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == int(np.prod(self.grid.shape))
        _check(self.grid.ctx.h, capi.lib().xf_vec_download(self.h, capi._ptr(out)))
        return out

    def assign(self, other):
        _check(self.grid.ctx.h, capi.lib().xf_vec_assign(self.h, other.h))
        return self

    def fill(self, c):
        _check(self.grid.ctx.h, capi.lib().xf_vec_fill(self.h, float(c)))
        return self

    def dot(self, other):
        out = C.c_double()
        _check(self.grid.ctx.h, capi.lib().xf_dot(self.h, other.h, C.byref(out)))
        return out.value

    def norm(self):
        out = C.c_double()
        _check(self.grid.ctx.h, capi.lib().xf_norm(self.h, C.byref(out)))
        return out.value

    def absmax(self):
        out, idx = C.c_double(), C.c_int64()
        _check(self.grid.ctx.h, capi.lib().xf_absmax(self.h, C.byref(out), C.byref(idx)))
        return out.value, idx.value

    def lincomb(self, p1, s1, p2=0.0, s2=None):
        _check(self.grid.ctx.h, capi.lib().xf_lincomb(float(p1), s1.h, float(p2), s2.h if s2 is not None else None,
                                                      self.h))
        return self

    def close(self):
        if self.h:
            if self.grid.h and self.grid.ctx.h:
                capi.lib().xf_vec_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Operator(_Owned):
    def __init__(self, grid, kind=XF_OP_LAPLACE, density=None):
        self.grid, self.kind = grid, kind
        h = C.c_void_p()
        _check(grid.ctx.h, capi.lib().xf_op_create(grid.h, kind, C.byref(h)))
        self.h = h
        grid._adopt(self)
        if density is not None:
            self.set_density(density)

    def set_density(self, rho):
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        _check(self.grid.ctx.h, capi.lib().xf_op_set_density(self.h, capi._ptr(rho)))

    def set_advection(self, u, v, w, tau, diff_coef, flags=XF_ADV_CONVECTIVE | XF_ADV_DIFFUSIVE):
        """XF_OP_ADVDIFF coefficients: advecting velocity Vecs (or None), tau, D, flags."""
        hh = [x.h if x is not None else None for x in (u, v, w)]
        _check(self.grid.ctx.h, capi.lib().xf_op_set_advection(self.h, *hh, float(tau), float(diff_coef), int(flags)))

    def set_diffusion_field(self, d):
        """XF_OP_ADVDIFF: per-cell diffusion coefficient Vec (the visTr form, XProblem.cpp:3204); None: the
        constant again."""
        _check(self.grid.ctx.h, capi.lib().xf_op_set_diffusion_field(self.h, _h(d)))

    def apply(self, x, y, s=None, sign=0, flags=0, w=None, want_dot=False):
        d = C.c_double()
        _check(self.grid.ctx.h, capi.lib().xf_matvec(self.h, x.h, y.h, s.h if s is not None else None, sign, flags,
                                                     w.h if w is not None else None,
                                                     C.byref(d) if want_dot else None))
        return d.value if want_dot else None

    def dot_op(self, x, y):
        out = C.c_double()
        _check(self.grid.ctx.h, capi.lib().xf_dot_op(self.h, x.h, y.h, C.byref(out)))
        return out.value

    def close(self):
        if self.h:
            if self.grid.h and self.grid.ctx.h:
                capi.lib().xf_op_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PackedOperator(Operator):
    """T1dPackOperator (XOperator.cpp:1135-1571) built on the GPU from `op`."""

    def __init__(self, op):
        self.grid, self.kind = op.grid, capi.XF_OP_PACK
        h = C.c_void_p()
        _check(op.grid.ctx.h, capi.lib().xf_pack_create(op.h, C.byref(h)))
        self.h = h
        op.grid._adopt(self)

    def transpose(self):
        """operator~ (XOperator.h:330): apply A^T from now on (again: A)."""
        _check(self.grid.ctx.h, capi.lib().xf_op_transpose(self.h))
        return self

    def size(self):
        r, a, t = C.c_int64(), C.c_int64(), C.c_int64()
        _check(self.grid.ctx.h, capi.lib().xf_pack_size(self.h, C.byref(r), C.byref(a), C.byref(t)))
        return r.value, a.value, t.value

    def csr(self, transpose=False):
        rows, nnz, nnz_t = self.size()
        m = nnz_t if transpose else nnz
        ptr, cols, vals = np.zeros(rows + 1, np.int32), np.zeros(m, np.int32), np.zeros(m)
        _check(self.grid.ctx.h, capi.lib().xf_pack_download(self.h, int(transpose), capi._ptr(ptr), capi._ptr(cols),
                                                            capi._ptr(vals)))
        return ptr, cols, vals


def solve_opts(method=XF_CG, precision=XF_PREC_FP64, rtol=1e-8, atol=0.0, maxit=100000, replace_every=50,
               check_every=16, exact=False, precond=None, cheb_ratio=0, cheb_degree=0):
    """precond: capi.XF_PRECOND_CHEB with XF_CG and XF_PREC_MIXED for the polynomial preconditioner
    (cheb_ratio: its lambda_max / lambda_min, 0 for the default; cheb_degree: even, 2 to 12, 0 for the
    default 8)."""
    o = capi.SolveOpts()
    capi.lib().xf_solve_opts_default(C.byref(o))
    o.method, o.precision, o.rtol, o.atol, o.maxit = method, precision, rtol, atol, maxit
    o.replace_every, o.check_every, o.exact = replace_every, check_every, int(exact)
    if precond is not None:
        o.precond = precond
    o.reserved[1] = int(cheb_ratio)
    o.reserved[2] = int(cheb_degree)
    return o


def solve(op, x, b, **kw):
    """Solve A x = b in place (x holds the initial guess); returns the stats."""
    o = solve_opts(**kw)
    st = capi.SolveStats()
    _check(op.grid.ctx.h, capi.lib().xf_solve(op.h, C.byref(o), x.h, b.h, C.byref(st)))
    return st


CG_KERNELS = ("stencil_f32", "xr_update_f32", "p_update_f32", "residual_f64", "stencil_f64", "pq_fused_f32",
              "pq_march_f32", "poly2_f32", "polyr_f32", "cheb_first_fused_f32", "cheb_last_f32",
              "cheb_middle_f32", "tl_prolong_ay_f32", "tl_first_f32", "tl_last_f32")


def selftest_division(ctx, n=1 << 24, seed=1):
    """Pairs (of n) where the time-step passes' reciprocal-based division differs from the IEEE one."""
    m = C.c_longlong()
    _check(ctx.h, capi.lib().xf_selftest_division(ctx.h, int(n), int(seed), C.byref(m)))
    return m.value


def voxelize_mesh(ctx, codes, x_nodes, y_nodes, z_nodes, vertices, faces, inside_code):
    """A copy of the point-code box with every point inside the closed triangle surface set to inside_code."""
    out = np.ascontiguousarray(codes, dtype=np.int32).copy()
    n1, n2, n3 = out.shape
    xs, ys, zs = (np.ascontiguousarray(a, dtype=np.float64) for a in (x_nodes, y_nodes, z_nodes))
    assert xs.size == n1 and ys.size == n2 and zs.size == n3
    v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
    f = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
    _check(ctx.h, capi.lib().xf_voxelize_mesh(ctx.h, n1, n2, n3, capi._ptr(xs), capi._ptr(ys), capi._ptr(zs),
                                              capi._ptr(v), v.shape[0], capi._ptr(f), f.shape[0], int(inside_code),
                                              capi._ptr(out)))
    return out


def cheb_factors(lmax, ratio, degree):
    """The polynomial preconditioner's factors as the solver builds them (host only): degree 2 gives one row
    (a0, a1, a2) of Horner coefficients, degree 2m gives m rows (1, b1, b2) of quadratic factors."""
    m = 1 if degree == 2 else degree // 2
    out = (C.c_float * (3 * m))()
    st = capi.lib().xf_cheb_factors_host(float(lmax), float(ratio), int(degree), out)
    if st != capi.XF_OK:
        raise XFError(st, f"no real quadratic factors for degree {degree}, ratio {ratio}")
    return np.array(list(out), dtype=np.float64).reshape(m, 3)


def profile_cg_kernels(op, reps=20):
    """Average ms per launch of each CG-iteration kernel, timed alone
    (pq_fused_f32 is absent where the grid does not take the fused path)."""
    out = (C.c_double * len(CG_KERNELS))()
    _check(op.grid.ctx.h, capi.lib().xf_profile_cg_kernels(op.h, int(reps), out))
    return {k: v for k, v in zip(CG_KERNELS, list(out)) if v >= 0}


def solve_host(op, x_host, b_host, **kw):
    """Host-buffer solve (upload, solve, download inside one C-ABI call)."""
    o = solve_opts(**kw)
    st = capi.SolveStats()
    _check(op.grid.ctx.h, capi.lib().xf_solve_host(op.h, C.byref(o), capi._ptr(x_host), capi._ptr(b_host),
                                                   C.byref(st)))
    return st


class SLAE:
    """TSLAE (XSLAE.h:9-48): holds A, x, b; SolveBy*() writes Result.

    Unlike the reference, the operands stay owned by the caller."""

    def __init__(self, A, x, b):
        self.A, self.x, self.b = A, x, b
        self.stats = None

    def UpdateP(self, p):      # XSLAE.cpp:37-40
        self.x.assign(p)

    def UpdateRP(self, rp):    # XSLAE.cpp:43-46
        self.b.assign(rp)

    def _run(self, method, **kw):
        self.stats = solve(self.A, self.x, self.b, method=method, **kw)
        if self.stats.status != capi.XF_OK:
            raise XFError(self.stats.status, capi.lib().xf_status_string(self.stats.status).decode())
        return self.stats

    def SolveByConjugateGradients(self, **kw):
        return self._run(XF_CG_REFERENCE, **kw)

    def SolveByBiConjugateGradientsStab(self, **kw):
        return self._run(XF_BICGSTAB, **kw)

    def SolveByMinimalResiduals(self, **kw):
        return self._run(XF_MINRES, **kw)

    def SolveByBiConjugateGradients(self, **kw):
        """Needs A packed (PackedOperator): the reference's BiCG applies A^T."""
        return self._run(XF_BICG, **kw)

    @staticmethod
    def SolveByScalarRunning(ctx, M, u, a, b, c, f, lines=(1, 1, 0, 0), ms=1):
        """TSLAE::SolveByScalarRunning for a batch of lines (see thomas_lines)."""
        nl1, nl2, ls1, ls2 = lines
        thomas_lines(ctx, M, u, a, b, c, f, nl1, nl2, ls1, ls2, ms)

    @property
    def Result(self):
        return self.x


# ---------------------------------------------------------------------------
# Time-step passes around the pressure solve (XProblem.cpp:5474-5829)
def _h(v):
    return v.h if v is not None else None


def pressure_rhs(gp, u, v, w, tau, rhs, density=None, border=None):
    """rhs |= the reference's pressure right-hand side (XProblem.cpp:5474-5512)."""
    _check(gp.ctx.h, capi.lib().xf_pressure_rhs(gp.h, u.h, v.h, w.h, _h(density), float(tau), _h(border), rhs.h))
    return rhs


def velocity_correct(axis, vel_prev, p, tau, vel, density=None, border=None):
    """vel |= the projected velocity component `axis` (XProblem.cpp:5598-5777)."""
    _check(vel.grid.ctx.h, capi.lib().xf_velocity_correct(int(axis), vel_prev.h, p.h, _h(density), float(tau),
                                                          _h(border), vel.h))
    return vel


def transfer_rhs(f_prev, rp, tau, out):
    """out |= the implicit transfer equation's right-hand side: (1/tau) f_prev + rp on Actual points, rp on the
    border rows (XProblem.cpp:3192)."""
    _check(out.grid.ctx.h, capi.lib().xf_transfer_rhs(f_prev.h, rp.h, float(tau), out.h))
    return out


def border_recalc(vel, border=None):
    """PreDefined points of vel |= 2 border - their Actual neighbour (XProblem.cpp:2996-3003)."""
    _check(vel.grid.ctx.h, capi.lib().xf_border_recalc(_h(border), vel.h))
    return vel


def border_follow(vel, border, axis, side):
    """border |= on face (axis, side), the values of vel's Actual neighbours (a lagged zero-gradient face)."""
    _check(vel.grid.ctx.h, capi.lib().xf_border_follow(vel.h, border.h, int(axis), int(side)))
    return border


def outflow_convective(vel, border, axis, speed, tau):
    """border |= on the high face of `axis`, the Defined outlet values advanced by db/dt + speed db/dn = 0 and
    shifted so the outlet's flux equals the inlet's (a convective outflow with mass balance)."""
    _check(vel.grid.ctx.h, capi.lib().xf_outflow_convective(vel.h, border.h, int(axis), float(speed), float(tau)))
    return border


def divergence_max(gp, u, v, w):
    """(max |div u| over Actual cells, (i, j, k)) as the control balance (XProblem.cpp:5782-5829)."""
    val = C.c_double()
    ijk = np.zeros(3, np.int32)
    _check(gp.ctx.h, capi.lib().xf_divergence_max(gp.h, u.h, v.h, w.h, C.byref(val), capi._ptr(ijk)))
    return val.value, tuple(int(t) for t in ijk)


def momentum_rhs(axis, gc, u_prev, v_prev, w_prev, vis=None, border=None, force=None, out=None):
    """Momentum right-hand side of velocity equation `axis` on the component grid gc (XProblem.cpp:5088-5419):
    returns the Vecs (uTr, vTr, wTr, visTr, rp), reusing `out` when given."""
    out = out if out is not None else tuple(gc.vec(None) for _ in range(5))
    _check(gc.ctx.h, capi.lib().xf_momentum_rhs(int(axis), u_prev.h, v_prev.h, w_prev.h, _h(vis), _h(border),
                                                 _h(force), *(o.h for o in out)))
    return out


def conc_transfer(gc, u, v, w, inlet=None, out=None):
    """Transfer terms of the concentration equation on its grid gc (XProblem.cpp:5886-5935): returns the Vecs
    (uTr, vTr, wTr, rp), reusing `out` when given; inlet is the PreDefined inlet values on the face i = 0."""
    out = out if out is not None else tuple(gc.vec(None) for _ in range(4))
    _check(gc.ctx.h, capi.lib().xf_conc_transfer(gc.h, u.h, v.h, w.h, _h(inlet), *(o.h for o in out)))
    return out


# ---------------------------------------------------------------------------
# Field output (XProblem.cpp:6132-6345, 6545-6590)
def write_vtk(path, nodes, x, y, z, u, v, w, p, density, conc, vis):
    """The time loop's VTK legacy ASCII volume, formatted on the device; returns the file size."""
    xyz = [np.ascontiguousarray(a, np.float64) for a in (x, y, z)]
    n = C.c_int64()
    _check(nodes.ctx.h, capi.lib().xf_vtk_write(str(path).encode(), nodes.h, *(capi._ptr(a) for a in xyz), u.h, v.h,
                                                 w.h, p.h, density.h, conc.h, vis.h, C.byref(n)))
    return n.value


def format_fixed6(ctx, values):
    """b"".join(b"%f\\n" % v for v in values), formatted on the device."""
    v = np.ascontiguousarray(values, np.float64).ravel()
    n = C.c_int64()
    _check(ctx.h, capi.lib().xf_format_fixed6(ctx.h, capi._ptr(v), v.size, None, 0, C.byref(n)))
    buf = C.create_string_buffer(max(int(n.value), 1))
    _check(ctx.h, capi.lib().xf_format_fixed6(ctx.h, capi._ptr(v), v.size, buf, n.value, C.byref(n)))
    return buf.raw[:n.value]


def write_npy(path, vec):
    """NPY file of a Vec's box with cnpy's header."""
    _check(vec.grid.ctx.h, capi.lib().xf_npy_write(str(path).encode(), vec.h))


# ---------------------------------------------------------------------------
def thomas_lines(ctx, M, u, a, b, c, f, nl1, nl2, ls1, ls2, ms):
    """TSLAE::SolveByScalarRunning over nl1*nl2 lines at once (XSLAE.cpp:416-445).
    u, a, b, c, f are FP64 Vecs (or raw device pointers); element m of line
    (l1, l2) sits at l1*ls1 + l2*ls2 + m*ms.  Asynchronous on the context stream."""
    def ptr(v):
        return capi.lib().xf_vec_data(v.h) if isinstance(v, Vec) else v
    _check(ctx.h, capi.lib().xf_thomas_lines(ctx.h, int(M), int(nl1), int(nl2), int(ls1), int(ls2), int(ms),
                                             ptr(u), ptr(a), ptr(b), ptr(c), ptr(f)))


def box_lines(shape, axis):
    """(M, nl1, nl2, ls1, ls2, ms) of the lines of a C-order box along axis 1..3."""
    n1, n2, n3 = shape
    s1, s2 = n2 * n3, n3
    if axis == 1:
        return n1 - 1, n2, n3, s2, 1, s1
    if axis == 2:
        return n2 - 1, n1, n3, s1, 1, s2
    return n3 - 1, n1, n2, s1, s2, 1


class Markers(_Owned):
    """Immersed-boundary node list on the device (TImmersedBoundary nodes and
    the marker side of TImmersedBoundaryProblem, XProblem.cpp:8436-8894)."""

    def __init__(self, ctx, pos, ref, kind, nxt, prv, dist0, curv0, node_stiff, params):
        self.ctx = ctx
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        pos, ref, curv0 = f64(pos).reshape(-1, 3), f64(ref).reshape(-1, 3), f64(curv0).reshape(-1, 3)
        self.nn = len(pos)
        keep = (pos, ref, i32(kind), i32(nxt), i32(prv), f64(dist0), curv0, f64(node_stiff), f64(params))
        h = C.c_void_p()
        _check(ctx.h, capi.lib().xf_ib_create(ctx.h, self.nn, *[capi._ptr(a) for a in keep], C.byref(h)))
        self.h = h
        ctx._adopt(self)

    def get(self, field):
        out = np.empty(3 * self.nn, np.float64)
        _check(self.ctx.h, capi.lib().xf_ib_download(self.h, field, capi._ptr(out)))
        return out.reshape(self.nn, 3) if field == XF_IB_POS else out.reshape(3, self.nn)

    def set(self, field, a):
        a = np.ascontiguousarray(a, dtype=np.float64).ravel()
        assert a.size == 3 * self.nn
        _check(self.ctx.h, capi.lib().xf_ib_upload(self.h, field, capi._ptr(a)))

    def interpolate(self, velocity, h0, axis):
        h0 = np.ascontiguousarray(h0, dtype=np.float64)
        _check(self.ctx.h, capi.lib().xf_ib_interpolate(self.h, velocity.h, capi._ptr(h0), int(axis)))

    def update_position(self, axis, tau):
        _check(self.ctx.h, capi.lib().xf_ib_update_position(self.h, int(axis), float(tau)))

    def compute_forces(self, axis):
        _check(self.ctx.h, capi.lib().xf_ib_compute_forces(self.h, int(axis)))

    def spread(self, force, h0, axis):
        h0 = np.ascontiguousarray(h0, dtype=np.float64)
        _check(self.ctx.h, capi.lib().xf_ib_spread(self.h, force.h, capi._ptr(h0), int(axis)))

    def close(self):
        if self.h:
            if self.ctx.h:
                capi.lib().xf_ib_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Learned preconditioner (no counterpart in the reference)
UNET_LAYERS = (("enc0a", 16, 16), ("enc0b", 16, 16), ("enc1a", 16, 32), ("enc1b", 32, 32), ("mid_a", 32, 64),
               ("mid_b", 64, 64), ("dec1a", 96, 32), ("dec1b", 32, 32), ("dec0a", 48, 16), ("dec0b", 16, 16),
               ("out", 16, 16))


def unet_init_params(seed=0):
    """He-normal weights over each layer's real fan-in (input 1 channel for
    enc0a, output 1 channel for out), zero biases; the padding stays 0."""
    rng = np.random.Generator(np.random.PCG64(seed))
    parts = []
    for name, ci, co in UNET_LAYERS:
        ci_real = 1 if name == "enc0a" else ci
        w = rng.standard_normal((27, co, ci)) * np.sqrt(2.0 / (27 * ci_real))
        if name == "enc0a":
            w[:, :, 1:] = 0
        if name == "out":
            w[:, 1:, :] = 0
            w *= np.sqrt(0.5)   # no ReLU after the output layer
        parts += [w.ravel(), np.zeros(co)]
    return np.concatenate(parts).astype(np.float32)


class UNet(_Owned):
    """3-level 3-D U-Net preconditioner on a grid (interior dims multiple of 4)."""

    def __init__(self, grid, params=None, seed=0):
        self.grid = grid
        h = C.c_void_p()
        _check(grid.ctx.h, capi.lib().xf_unet_create(grid.h, C.byref(h)))
        self.h = h
        grid._adopt(self)
        n = C.c_int64()
        _check(grid.ctx.h, capi.lib().xf_unet_param_count(self.h, C.byref(n)))
        self.nparams = n.value
        self.set_params(unet_init_params(seed) if params is None else params)

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.nparams
        _check(self.grid.ctx.h, capi.lib().xf_unet_set_params(self.h, capi._ptr(p)))

    def params(self):
        p = np.zeros(self.nparams, np.float32)
        _check(self.grid.ctx.h, capi.lib().xf_unet_get_params(self.h, capi._ptr(p)))
        return p

    def grads(self):
        p = np.zeros(self.nparams, np.float32)
        _check(self.grid.ctx.h, capi.lib().xf_unet_get_grads(self.h, capi._ptr(p)))
        return p

    def apply(self, r, z):
        _check(self.grid.ctx.h, capi.lib().xf_unet_apply(self.h, r.h, z.h))
        return z

    def train_step(self, r, e, lr=1e-3, update=True, op=None):
        """One step on (r, e); with op one minus the A-norm cosine of output and error,
        else the MSE against e / rms e."""
        loss = C.c_double()
        _check(self.grid.ctx.h, capi.lib().xf_unet_train_step(self.h, op.h if op is not None else None, r.h, e.h,
                                                              float(lr), int(update), C.byref(loss)))
        return loss.value

    def close(self):
        if self.h:
            if self.grid.h and self.grid.ctx.h:
                capi.lib().xf_unet_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_fcg(op, x, b, unet=None, precond=None, rtol=1e-8, maxit=100000, window=8, degree=0, ratio=0,
              precision=XF_PREC_FP64):
    """Flexible CG, FCG(window), with the U-Net (default when given), Jacobi or no preconditioner.
    precond=XF_PRECOND_UNET2 with a U-Net built on the coarse grid of F^3 blocks (`workloads.coarse_grid`)
    runs the learned two-level preconditioner, in FP64 or (precision=XF_PREC_MIXED) with FP32 vectors and
    FP64 dots."""
    o = solve_opts(method=capi.XF_FCG, rtol=rtol, maxit=maxit)
    o.precision = int(precision)
    o.reserved[0] = int(window)
    o.reserved[1] = int(ratio)    # XF_PRECOND_UNET2: smoothing interval ratio (0: default)
    o.reserved[2] = int(degree)   # XF_PRECOND_UNET2: smoothing degree (0: default)
    o.precond = precond if precond is not None else (capi.XF_PRECOND_UNET if unet is not None else
                                                     capi.XF_PRECOND_NONE)
    st = capi.SolveStats()
    _check(op.grid.ctx.h, capi.lib().xf_solve_fcg(op.h, unet.h if unet is not None else None, C.byref(o), x.h, b.h,
                                                  C.byref(st)))
    return st


def harvest_pairs(op, b, iters, xstar=None):
    """(residual, error) pairs from plain FP64 CG's own iterates on A x = b:
    for each k in `iters`, x_k = CG after k iterations from 0, r_k = b - A x_k,
    e_k = x* - x_k with x* the converged (1e-10) solution.  Returns lists of
    device Vecs (r_k, e_k)."""
    g = op.grid
    if xstar is None:
        xstar = g.vec(np.zeros(g.shape))
        solve(op, xstar, b, method=XF_CG, rtol=1e-10)
    rs, es = [], []
    for k in iters:
        xk = g.vec(np.zeros(g.shape))
        solve(op, xk, b, method=XF_CG, rtol=1e-30, maxit=int(k))
        ax = g.vec(None)
        op.apply(xk, ax, flags=XF_ZERO_INACTIVE)
        r = g.vec(None).lincomb(1.0, b, -1.0, ax)
        e = g.vec(None).lincomb(1.0, xstar, -1.0, xk)
        rs.append(r)
        es.append(e)
    return rs, es
