/* xflow_gb300: GB300-native (sm_103a) pressure-projection path of xFlow.
 *
 * C ABI only: plain pointers, sizes and status codes; no C++ types and no
 * exceptions cross it.  One context owns one CUDA stream on one device and is
 * not thread-safe.  Every call returns XF_OK (0) or an XF_* status; on error
 * xf_last_error() holds a one-line reason.
 *
 * Data convention (identical to the reference): a grid of N x L x M intervals
 * has a box of n1 = N+1, n2 = L+1, n3 = M+1 cells, stored C-order with k
 * fastest, exactly the reference's double*** [i][j][k] flattened.  Point codes
 * are the reference's (XMask.h:6-7, XGrid.h:11, XOperator.h:13-18):
 *   0 Fictive, 1 Actual, 3 Defined, 4 PreDefined, 5 Normal, 6 PreNormal,
 *   7 Equation, 8 PreEquation.
 * Rn indices are 1-based in i->j->k order (XSpaceModel.cpp:383-406).
 *
 * Each entry point names the reference interface it replaces.
 */
#ifndef XFLOW_H
#define XFLOW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
enum {
  XF_OK = 0,
  XF_ERR_ARG = 1,        /* bad argument (null pointer, size mismatch)        */
  XF_ERR_CUDA = 2,       /* CUDA runtime error                                 */
  XF_ERR_MASK = 3,       /* a row the reference throws on (XOperator.cpp:1037, */
                         /* 1043-1055, 1075-1080, 1122) or would read outside  */
                         /* its arrays                                         */
  XF_ERR_NOMEM = 4,
  XF_ERR_STATE = 5,      /* object used with the wrong grid / dtype            */
  XF_ERR_UNSUPPORTED = 6,
  XF_ERR_CHECK = 7,      /* a border-condition consistency check of the        */
                         /* reference failed (XProblem.cpp:5690-5694, 5747-5752) */
  XF_STALL = 10,         /* solver made no progress                            */
  XF_DIVERGED = 11,
  XF_NAN = 12,
  XF_MAXIT = 13,         /* iteration cap reached (the reference has none)     */
  XF_BREAKDOWN = 14      /* zero denominator (XSLAE.cpp:274-275)               */
};

enum { XF_F64 = 0, XF_F32 = 1 };

/* Operators (XOperator.h:292-319, 410-423; XF_OP_PACK: T1dPackOperator,
 * XOperator.h:320-378, made by xf_pack_create; XF_OP_ADVDIFF: the implicit
 * advection-diffusion operator of the momentum / transport equations, set up
 * by xf_op_set_advection). */
enum { XF_OP_LAPLACE = 0, XF_OP_VARDIV = 1, XF_OP_PACK = 2, XF_OP_ADVDIFF = 3 };
/* xf_op_set_advection flags (THydrodynamicsProblem's flagConvective and
 * flagDiffusion, XProblem.cpp:1236-1238; XF_ADV_UPWIND: its first-order
 * upwind scheme, schemeType 1 of SolveTransferEquation_, XProblem.cpp:
 * 1828-1843, the concentration equation's) */
enum { XF_ADV_CONVECTIVE = 1, XF_ADV_DIFFUSIVE = 2, XF_ADV_UPWIND = 4 };

/* xf_matvec flags */
enum {
  XF_EXACT = 1,          /* FP64 only: the reference's operation order, bit-exact */
  XF_ZERO_INACTIVE = 2   /* write 0 to inactive cells instead of leaving them   */
};

typedef struct xf_ctx xf_ctx;
typedef struct xf_grid xf_grid;
typedef struct xf_vec xf_vec;
typedef struct xf_op xf_op;

/* ---- context ------------------------------------------------------------- */
int xf_create(int device, xf_ctx** out);
int xf_destroy(xf_ctx* ctx);
const char* xf_last_error(const xf_ctx* ctx);
const char* xf_status_string(int status);
int xf_synchronize(xf_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that order their own
 * work against it. */
void* xf_stream(xf_ctx* ctx);

/* ---- grid: T3dNormalGrid + TRnRelease3dSpaceModel ------------------------- */
/* Replaces T3dNormalGrid(sep1, sep2, sep3, mask, normals) (XGrid.h:282) and
 * TRnRelease3dSpaceModel(1, masks) (XSpaceModel.h:499-533, built as
 * XProblem.cpp:4116-4207 does).  codes: n1*n2*n3 int32; hx: n1-1 separations
 * (TSeparator::Separation), hy: n2-1, hz: n3-1; normals: 3 doubles per cell or
 * NULL, all-zero meaning no normal.  Host pointers. */
int xf_grid_create(xf_ctx* ctx, int n1, int n2, int n3, const int32_t* codes, const double* hx,
                   const double* hy, const double* hz, const double* normals, xf_grid** out);
int xf_grid_destroy(xf_grid* g);
/* TRnSpaceModel::EndIndex (XSpaceModel.h:50-54): number of active cells. */
int xf_grid_end_index(const xf_grid* g, int64_t* end_index);
/* Rn numbering (XSpaceModel.cpp:383-406), computed on the GPU: inv_box gets
 * the 1-based Rn index of each cell (0 when inactive), fwd_ijk 3 ints (i,j,k)
 * per Rn index.  Host pointers, either may be NULL. */
int xf_grid_rn_map(const xf_grid* g, int32_t* inv_box, int32_t* fwd_ijk);
/* Space mask 0/1 per cell (XProblem.cpp:4155-4182).  Host pointer. */
int xf_grid_space_mask(const xf_grid* g, uint8_t* smask_box);
/* Validity of the grid for an operator: XF_OK or XF_ERR_MASK with the first
 * offending cell (flat index) in bad_cell. */
int xf_grid_check(const xf_grid* g, int op, int64_t* bad_cell);

/* ---- vectors: TRnRelease3dSpace ------------------------------------------ */
/* Replaces TRnRelease3dSpace(model) (XSpace.h:595-633): a device box of the
 * grid's shape, zero-filled like TRnRelease3dData (XSpace.cpp:2213-2225). */
int xf_vec_create(xf_grid* g, int dtype, xf_vec** out);
int xf_vec_destroy(xf_vec* v);
int xf_vec_upload(xf_vec* v, const double* host_box);        /* whole box      */
int xf_vec_download(const xf_vec* v, double* host_box);      /* whole box      */
/* TSpace::Assign (XSpace.cpp:2343-2361): whole-box copy (dtypes may differ). */
int xf_vec_assign(xf_vec* dst, const xf_vec* src);
/* x |= c on active cells (XSpace.cpp:2424-2487 for c = 0). */
int xf_vec_fill(xf_vec* v, double c);
/* Raw device pointer of the box (double* or float*). */
void* xf_vec_data(xf_vec* v);

/* ---- operators ----------------------------------------------------------- */
/* T3dLaplaceOperator (XOperator.cpp:809-1129) or
 * T3dVariableDivergentedOperator (XOperator.cpp:1901-2293). */
int xf_op_create(xf_grid* g, int kind, xf_op** out);
int xf_op_destroy(xf_op* op);
/* T3dVariableDivergentedOperator::withDensity (XOperator.cpp:2235-2268):
 * copies the density box (host pointer, n1*n2*n3 doubles). */
int xf_op_set_density(xf_op* op, const double* host_density_box);

/* Coefficients of an XF_OP_ADVDIFF operator.  Replaces the ADI line systems of
 * the transfer / momentum equations (THydrodynamicsProblem, XProblem.cpp:
 * 1236-1238 and the same coefficients at :3199-3218), which the reference
 * solves direction by direction with TSLAE::SolveByScalarRunning, by one
 * implicit 7-point operator: the sum over the three directions of the
 * reference's line coefficients.  On Actual cells, with per direction
 * h_1 = h[m-1], h = h[m], hx2 = h_1 + h, hxhxh = h_1 h (h_1 + h) / 2 and the
 * advecting velocity component vd at the cell,
 *   A_d = conv 0.5 (-vd / hx2) + diff 0.5 (-D h / hxhxh)      (f[m-1])
 *   B_d = diff 0.5 D hx2 / hxhxh                              (f[m])
 *   C_d = conv 0.5 (vd / hx2) + diff 0.5 (-D h_1 / hxhxh)     (f[m+1])
 *   (A f)_c = (1/tau) f_c + sum_d (A_d f[m-1] + B_d f_c + C_d f[m+1]),
 * in that evaluation order with XF_EXACT (FP64).  Without it, FP64 rows read
 * a table of seven coefficients per cell (the centre 1/tau + B_x + B_y + B_z
 * and the six neighbours'), built once after each xf_op_set_advection /
 * xf_op_set_diffusion_field, and apply them by FMAs: within a few units in
 * the last place of the exact rows, at 7 FP64 operations a row instead of
 * 19 and 15 divisions.  With XF_ADV_UPWIND the convective part takes
 * the upstream neighbour over h (vd < 0: B_d += conv 0.5 (-vd / h),
 * C_d += conv 0.5 (vd / h); else A_d += conv 0.5 (-vd / h),
 * B_d += conv 0.5 (vd / h)); B_d is the convective term plus the diffusive
 * one, in that order.  PreDefined and PreNormal rows are the Laplace
 * operator's (semi-sum, normal derivative).  u, v, w are FP64 boxes of the
 * operator's grid (NULL: 0), copied into the operator; flags are
 * XF_ADV_CONVECTIVE | XF_ADV_DIFFUSIVE | XF_ADV_UPWIND.  Nonsymmetric: solve it with
 * XF_BICGSTAB, XF_MINRES, or XF_BICG on its packed form. */
int xf_op_set_advection(xf_op* op, const xf_vec* u, const xf_vec* v, const xf_vec* w, double tau,
                        double diff_coef, int flags);
/* Variable-viscosity form (the visTr overload of SolveTransferEquation__,
 * XProblem.cpp:2784-3420, diffCoefVar[i][j][k] at :3204): d, an FP64 box of
 * the operator's grid, is copied and replaces diff_coef cell by cell; NULL
 * returns to the constant. */
int xf_op_set_diffusion_field(xf_op* op, const xf_vec* d);

/* Packed operator: replaces T1dPackOperator(model, A, &null) (XOperator.cpp:
 * 1135-1350) built from A (Laplace or variable-density, density set).  Rows
 * and columns are the Rn indices of A's grid; row i holds the nonzero A[i][c]
 * for c over the cell and its space neighbours at i-1, i+1, j-1, j+1, k-1, k+1
 * (the activity table, XOperator.cpp:837-936), in that order; the transposed
 * storage likewise per column.  Values are A's own FP64 arithmetic, bit for
 * bit.  The result is an xf_op of kind XF_OP_PACK over the same grid: xf_matvec
 * applies the row dot in storage order (XOperator.cpp:1550-1571, FP64 only),
 * xf_solve accepts it with every FP64 method, and XF_BICG requires it.  A zero
 * row or column returns XF_ERR_MASK (the reference throws, :1233, :1316). */
int xf_pack_create(xf_op* a, xf_op** out);
/* T1dPackOperator::operator~ (XOperator.h:330): switch between A and A^T.
 * Other operators return XF_ERR_UNSUPPORTED (the reference throws,
 * XOperator.h:302). */
int xf_op_transpose(xf_op* op);
/* Rows (= EndIndex) and nonzeros of the row and column storages. */
int xf_pack_size(const xf_op* pack, int64_t* rows, int64_t* nnz, int64_t* nnz_t);
/* The row (transpose = 0) or column (1) storage as 0-based CSR over Rn: ptr
 * rows+1 entries, cols/vals nnz entries.  Host pointers. */
int xf_pack_download(const xf_op* pack, int transpose, int32_t* ptr, int32_t* cols, double* vals);

/* y |= A(x) + sign*s  (sign 0, +1, -1; s may be NULL for sign 0), on active
 * cells: TRnRelease3dSpace::LocalReleaseAssignSpeedLinearCombination(op)
 * (XSpace.cpp:3013-3217).  Inactive cells of y are left as they are, or set
 * to 0 with XF_ZERO_INACTIVE.  With opt_dot non-NULL also returns (w, y) over
 * active cells for w = opt_w (or x when opt_w is NULL) in FP64. */
int xf_matvec(xf_op* op, const xf_vec* x, xf_vec* y, const xf_vec* s, int sign, int flags,
              const xf_vec* opt_w, double* opt_dot);

/* ---- vector algebra: TRnRelease3dSpace masked loops ---------------------- */
/* z |= p1*s1 + p2*s2 on active cells (XSpace.cpp:2489-3010); s2 may be NULL. */
int xf_lincomb(double p1, const xf_vec* s1, double p2, const xf_vec* s2, xf_vec* z);
/* (a, b) over active cells, FP64 (XSpace.cpp:3261-3342). */
int xf_dot(const xf_vec* a, const xf_vec* b, double* out);
/* TNormalizedSpace::Norma: sqrt of the masked sum of squares
 * (XSpace.cpp:3219-3259, 1205-1217). */
int xf_norm(const xf_vec* a, double* out);
/* (x, A y) (XSpace.cpp:3344-3419). */
int xf_dot_op(xf_op* op, const xf_vec* x, const xf_vec* y, double* out);
/* GetAbsMaxElement(index) (XSpace.cpp:3428-3487, type 1): the first strict
 * maximum of |a| in i->j->k order and its Rn index (1 when all are 0). */
int xf_absmax(const xf_vec* a, double* out, int64_t* rn_index);

/* ---- solvers: TSLAE ------------------------------------------------------- */
enum {
  XF_CG = 0,             /* Hestenes-Stiefel CG, relative tolerance (the FP64 baseline)*/
  XF_CG_REFERENCE = 1,   /* TSLAE::SolveByConjugateGradients, XSLAE.cpp:56-157     */
  XF_BICGSTAB = 2,       /* TSLAE::SolveByBiConjugateGradientsStab, :667-768       */
  XF_MINRES = 3,         /* TSLAE::SolveByMinimalResiduals, :350-414               */
  XF_BICG = 4,           /* TSLAE::SolveByBiConjugateGradients, :159-348 (packed   */
                         /* operators only: it needs A^T)                        */
  XF_FCG = 5             /* flexible CG with a preconditioner                      */
};
enum { XF_PREC_FP64 = 0, XF_PREC_MIXED = 1 };
/* XF_PRECOND_CHEB: XF_CG with XF_PREC_MIXED on a uniform Laplace grid without
 * boundary rows, preconditioned by z = p(A) r, p the polynomial of `degree`
 * Chebyshev-iteration steps over [lambda_max / ratio, lambda_max]
 * (lambda_max the Gershgorin bound; degree = opts.reserved[2], even, 2 to 12,
 * default 8; ratio = opts.reserved[1], default 30 for degree 2, 120 for
 * degree 4 and 250 above).  Degree 2 applies both stencil levels in one pass
 * over memory; degree 2 m is the product of m real quadratic factors, one
 * pass each. */
/* XF_PRECOND_UNET2: xf_solve_fcg with the network as the coarse solver of a
 * two-level preconditioner (no counterpart in the reference).  The network is
 * built on a coarse grid whose interior cells are F x F x F blocks of the
 * operator's interior (F >= 2, equal on every axis); with P the
 * piecewise-constant prolongation over the blocks, y = P U-Net(P^T r),
 * omega = (y, r) / (y, A y) and z = omega y + s p(A) (r - omega A y), p the
 * XF_PRECOND_CHEB polynomial (FP32 passes; degree opts.reserved[2], default
 * 8; ratio opts.reserved[1], default 60) scaled by s so that
 * lambda s p(lambda) is closest to 1 on its interval.  Uniform Laplace grids
 * without boundary rows. */
/* XF_PRECOND_JACOBI: with xf_solve_fcg, the Laplace diagonal; with
 * XF_BICGSTAB on an XF_OP_LAPLACE or XF_OP_ADVDIFF operator, right
 * preconditioning by the inverse row diagonals (the Actual rows' diagonals,
 * the border rows' own): the residual and the stop rule stay those of
 * A x = b, and rows of very different scales (semi-sums of 1/2, normal
 * differences of 1/h, Actual rows of 1/h^2 or 1/tau) no longer slow the
 * iteration down. */
enum { XF_PRECOND_NONE = 0, XF_PRECOND_JACOBI = 1, XF_PRECOND_UNET = 2, XF_PRECOND_CHEB = 3, XF_PRECOND_UNET2 = 4 };
/* Host only (no device work): the XF_PRECOND_CHEB polynomial as the solver
 * builds it, in powers of A.  degree 2 writes its three Horner coefficients
 * (a0, a1, a2: z = a0 r + A (a1 r + a2 A r)); degree 2m (4 to 12) writes m
 * real quadratic factors (1, b1, b2), p = p_1 ... p_m, 3m floats.  Every
 * form is scaled so that p(0) = 1.  XF_ERR_ARG when the roots do not pair
 * into real factors that reproduce p. */
int xf_cheb_factors_host(double lmax, double ratio, int degree, float* factors);

typedef struct {
  int method;            /* XF_CG ...                                              */
  int precision;         /* XF_PREC_FP64 or XF_PREC_MIXED (CG; FCG + UNET2)        */
  int precond;           /* XF_PRECOND_*                                           */
  int maxit;             /* iteration cap; 0 = 100000                              */
  double rtol;           /* relative tolerance on ||b - A x||_2 / ||b||_2 (XF_CG,  */
                         /* XF_FCG, mixed); <= 0 means 1e-8                        */
  double atol;           /* absolute tolerance of the reference-semantics methods; */
                         /* <= 0 means the reference's hard-coded value            */
  int replace_every;     /* mixed: true-residual replacement period (50)           */
  int check_every;       /* host polls the device convergence flag every this     */
                         /* many iterations (16)                                   */
  int exact;             /* reference-semantics methods: use XF_EXACT matvecs      */
  int reserved[7];
} xf_solve_opts;

typedef struct {
  int status;            /* XF_OK or XF_MAXIT / XF_BREAKDOWN / XF_NAN / XF_STALL   */
  int iterations;        /* inner (Krylov) iterations                              */
  int replacements;      /* mixed: true-residual replacements done                 */
  int fallbacks;         /* FCG: times it fell back to plain CG                    */
  double rel_resid;      /* final true ||b - A x||_2 / ||b||_2, FP64               */
  double abs_resid;      /* final value the method's own stopping rule tested      */
  double ms;             /* device time of the solve                               */
  double reserved[4];    /* [0]: kernels launched (mixed CG, mixed FCG)            */
} xf_solve_stats;

void xf_solve_opts_default(xf_solve_opts* o);
/* TSLAE(A, x, b) + SolveBy*() + Result (XSLAE.h:12-35): x holds the initial
 * guess on entry (warm start as TSLAE::UpdateP, XSLAE.cpp:37-40) and the
 * result on exit.  x and b are FP64 vectors of op's grid. */
int xf_solve(xf_op* op, const xf_solve_opts* opts, xf_vec* x, const xf_vec* b, xf_solve_stats* stats);
/* The same with host boxes (upload b and x, solve, download x): the call a
 * host-resident caller such as the reference's time loop makes.  The
 * operator keeps the two device boxes between calls (released by
 * xf_op_destroy), so calls on one operator must not overlap. */
int xf_solve_host(xf_op* op, const xf_solve_opts* opts, double* host_x, const double* host_b,
                  xf_solve_stats* stats);

/* ---- voxelisation ----------------------------------------------------------- */
/* Sets codes[(i n2 + j) n3 + k] = inside_code for every point (x_nodes[i],
 * y_nodes[j], z_nodes[k]) inside the closed triangle surface (vertices: 3
 * doubles each; faces: 3 vertex indices each), leaving the other codes as
 * they are.  The planned boundary's voxeliser for the immersed-body
 * configuration; no counterpart in the reference, which uses the STL
 * vertices only as markers (XImmersedBoundary.cpp:1560-1570).  Parity of
 * crossings along x with the rasterisation top-left rule on shared edges.
 * XF_ERR_ARG for a face naming a vertex out of range or a ray crossing the
 * surface more than 128 times.  codes is a host box. */
int xf_voxelize_mesh(xf_ctx* ctx, int n1, int n2, int n3, const double* x_nodes, const double* y_nodes,
                     const double* z_nodes, const double* vertices, long long nvert, const int32_t* faces,
                     long long nface, int32_t inside_code, int32_t* codes);

/* ---- time-step passes around the pressure solve --------------------------- */
/* TVPProblem::SolveBySplitting (XProblem.cpp:5474-5829).  Staggered boxes as
 * the reference's grids (XStatement.h:127-135): for a pressure grid gp of
 * n1 x n2 x n3, u lives on an (n1-1) x n2 x n3 grid, v on n1 x (n2-1) x n3 and
 * w on n1 x n2 x (n3-1); each is an FP64 xf_vec of its own xf_grid, whose
 * point codes and separations (hxU, hyV, hzW) the passes read.  density is an
 * FP64 pressure box (NULL: 1 everywhere); border boxes hold the boundary
 * values the reference's GetBorderCondition* return (NULL: 0).  Results are
 * bit-identical to the reference's loops.  A cell the reference throws on
 * returns XF_ERR_MASK (or XF_ERR_CHECK for its value checks), naming the first
 * such cell in its loop order. */
/* Right-hand side of the implicit transfer equation that replaces the ADI
 * sweeps of one velocity component (SolveTransferEquation__, XProblem.cpp:
 * 5421, 2784-3420; solved with XF_OP_ADVDIFF): out = (1/tau) f_prev + rp on
 * Actual points (the line systems' base term, XProblem.cpp:3192), rp on the
 * other active points (border rows: rp holds the border value
 * xf_momentum_rhs put there), f_prev on inactive points.  FP64 boxes of one
 * velocity grid. */
int xf_transfer_rhs(const xf_vec* f_prev, const xf_vec* rp, double tau, xf_vec* out);
/* After that solve, the sector ends as the reference's ADI sweeps recalculate
 * them (XProblem.cpp:2975-3003): every Defined point with an Actual neighbour
 * takes its border value, and every PreDefined point becomes 2 border - (its
 * one Actual neighbour), so the border rows hold (exactly, and to rounding)
 * before xf_velocity_correct checks them.  XF_ERR_MASK for a PreDefined point with
 * no or several Actual neighbours (the reference's throws). */
int xf_border_recalc(const xf_vec* border, xf_vec* vel);
/* A zero-gradient (outflow) face for a time loop: each PreDefined point of vel's
 * grid on face (axis 1..3, side 0 low / 1 high) gets, in border, the current
 * value of its Actual neighbour across the face; the next step's semi-sum row
 * then makes the face value follow the interior (lagged by one step).  No
 * counterpart in the reference, whose border values come from its statement's
 * GetBorderCondition* hooks. */
int xf_border_follow(const xf_vec* vel, xf_vec* border, int axis, int side);
/* A convective outflow for a time loop, on the high face of `axis` (1..3) of
 * vel's grid for the component normal to that face (its Defined points): each
 * border value b takes one explicit upwind step of db/dt + speed db/dn = 0,
 * b' = b - (speed tau / h) (b - v_a), h the spacing across the face and v_a
 * the point's neighbour inside; then all of them shift by one amount so that
 * the outlet's area-weighted sum equals the inlet's (the Defined points of the
 * low face), which keeps an all-Neumann pressure system consistent.  Areas
 * are the products of the face cells' widths.  No counterpart in the
 * reference, whose border values come from its statement's hooks.  FP64
 * vectors of one velocity grid; one block, deterministic. */
int xf_outflow_convective(const xf_vec* vel, xf_vec* border, int axis, double speed, double tau);
/* Pressure right-hand side (XProblem.cpp:5474-5512): Fictive 0; Actual
 * -(rho^2 du/dx + dv/dy + dw/dz) / tau; PreDefined the border value. */
int xf_pressure_rhs(const xf_grid* gp, const xf_vec* u, const xf_vec* v, const xf_vec* w, const xf_vec* density,
                    double tau, const xf_vec* border, xf_vec* rhs);
/* Velocity correction of component `axis` (XProblem.cpp:5598-5777):
 * vel = vel_prev - tau dp/dx_axis / rho on Actual/Normal/Equation cells, the
 * border value on Defined cells, then PreDefined cells mirror their single
 * Actual neighbour (2 * border - vel[neighbour]).  p is the pressure box. */
int xf_velocity_correct(int axis, const xf_vec* vel_prev, const xf_vec* p, const xf_vec* density, double tau,
                        const xf_vec* border, xf_vec* vel);
/* Control balance (XProblem.cpp:5782-5829): the first strict maximum of
 * |div u| over Actual pressure cells in i->j->k order, and its (i, j, k)
 * (-1s when no cell beats 0). */
int xf_divergence_max(const xf_grid* gp, const xf_vec* u, const xf_vec* v, const xf_vec* w, double* value,
                      int32_t* ijk);
/* Momentum right-hand side of velocity equation `axis` (1 u, 2 v, 3 w),
 * TVPProblem::SolveBySplitting XProblem.cpp:5088-5419, on the component's own
 * grid (the grid of the five outputs, distinct FP64 vectors):
 *  - Actual cells: the transfer velocities averaged onto the component's
 *    nodes (4-point means of the other two components, :5108-5133), the face
 *    viscosity (mean of the two pressure-box values of vis straddling the
 *    node), rp = force (GetForce: the immersed-boundary forcing, NULL = 0),
 *    then rp += dVis . (dVel + dU), central differences of those fields
 *    (:5352-5419);
 *  - Defined and PreDefined cells (and, for axis 1, Normal cells whose normal
 *    is along x only): zero transfer fields, rp = border;
 *  - Fictive cells: all zero.
 * u_prev, v_prev, w_prev are the staggered boxes of the pressure box one layer
 * longer than the component along `axis`; vis is that pressure box (NULL: 0);
 * border and force are component boxes (NULL: 0).  Cells the reference throws
 * on (Equation, PreNormal, PreEquation, other Normal cells, unknown codes, an
 * Actual cell on the box face) return XF_ERR_MASK naming the first in its loop
 * order.  Bit-identical to the reference's loops (FP64, no contraction). */
int xf_momentum_rhs(int axis, const xf_vec* u_prev, const xf_vec* v_prev, const xf_vec* w_prev, const xf_vec* vis,
                    const xf_vec* border, const xf_vec* force, xf_vec* u_tr, xf_vec* v_tr, xf_vec* w_tr,
                    xf_vec* vis_tr, xf_vec* rp);

/* Transfer terms of the concentration equation (TVPProblem::SolveBySplitting,
 * XProblem.cpp:5886-5935) on the concentration grid gc (the pressure box):
 *  - Actual points: u_tr = (u[i-1] + u[i]) / 2, v_tr and w_tr likewise from
 *    the staggered boxes, rp = 0;
 *  - PreDefined points: zero velocities, rp = inlet on the face i = 0
 *    (ConcentrationInletCondition; inlet NULL: 0), 0 elsewhere;
 *  - Fictive and PreNormal points: all zero.
 * The outputs are distinct FP64 vectors of gc; u, v, w the staggered boxes.
 * Defined, Normal, Equation and PreEquation points (the reference's throws),
 * unknown codes and Actual points on the box face return XF_ERR_MASK naming
 * the first in its loop order.  Bit-identical to the reference's loop.  The
 * equation itself is XF_OP_ADVDIFF with XF_ADV_CONVECTIVE | XF_ADV_UPWIND
 * (and XF_ADV_DIFFUSIVE for a nonzero coefficient), right-hand side
 * xf_transfer_rhs(c_prev, rp, tau). */
int xf_conc_transfer(const xf_grid* gc, const xf_vec* u, const xf_vec* v, const xf_vec* w, const xf_vec* inlet,
                     xf_vec* u_tr, xf_vec* v_tr, xf_vec* w_tr, xf_vec* rp);

/* ---- field output ----------------------------------------------------------- */
/* VTK legacy ASCII volume of one time step, replacing the writer in
 * TVPProblem::SolveBySplitting (XProblem.cpp:6132-6345), byte for byte:
 * header, POINTS (node coordinates x[i], y[j], z[k] for node indices 1..N-1,
 * 1..L-1, 1..M-1, k outermost), the velocity averaged from the staggered
 * boxes onto the nodes (0 at Fictive nodes of `nodes`), then pressure,
 * density, concentration and viscosity averaged over the 8 surrounding
 * pressure-box cells (sum of all 8 over the count of non-Fictive ones in the
 * field's own grid; viscosity counts with the concentration grid, as the
 * reference does), every number as C's "%f" prints it.  nodes is the node
 * grid, box (N+1) x (L+1) x (M+1); x, y, z host arrays of N+1, L+1, M+1
 * coordinates; u, v, w the staggered boxes and p, density, conc, vis FP64
 * vectors on their grids, box (N+2) x (L+2) x (M+2).  The text is formatted
 * on the device and streamed to `path`; *bytes (optional) receives the file
 * size.  Synchronous. */
int xf_vtk_write(const char* path, const xf_grid* nodes, const double* x, const double* y, const double* z,
                 const xf_vec* u, const xf_vec* v, const xf_vec* w, const xf_vec* p, const xf_vec* density,
                 const xf_vec* conc, const xf_vec* vis, int64_t* bytes);
/* "%f\n" of each of n host values, formatted on the device (the VTK
 * writer's number formatting): *length receives the byte count; the text is
 * stored into out when capacity allows (out may be NULL to query). */
int xf_format_fixed6(xf_ctx* ctx, const double* values, int64_t n, char* out, int64_t capacity, int64_t* length);
/* NPY file of a vector's box, shape (n1, n2, n3), '<f8' or '<f4', C order,
 * with the header cnpy::npy_save writes (cnpy.h:66-112, 206-233; the time
 * loop's NPY output, XProblem.cpp:6545-6590).  Synchronous. */
int xf_npy_write(const char* path, const xf_vec* vec);

/* ---- tridiagonal lines ---------------------------------------------------- */
/* Replaces TSLAE::SolveByScalarRunning(M, u, a, b, c, f) (XSLAE.h:23,
 * XSLAE.cpp:416-445), called once per grid line by the ADI sweeps
 * (XProblem.cpp:1369, 2049, 2734, 3427): here every line of a sweep in one
 * call.  Solves a[m] u[m-1] + b[m] u[m] + c[m] u[m+1] = f[m], m = 1..M-1, with
 * u[0] and u[M] given (and kept), for nl1 * nl2 lines; element m of line
 * (l1, l2) of every array is at offset l1*ls1 + l2*ls2 + m*ms.  All arrays are
 * FP64 device memory (e.g. xf_vec_data of boxes).  The reference's recurrences
 * and operation order: bit-identical results.  Asynchronous on the context
 * stream; uses a context workspace of M * nl1 * nl2 doubles. */
int xf_thomas_lines(xf_ctx* ctx, int M, int nl1, int nl2, int64_t ls1, int64_t ls2, int64_t ms, double* u,
                    const double* a, const double* b, const double* c, const double* f);

/* ---- immersed boundary ---------------------------------------------------- */
/* Replaces the marker side of TImmersedBoundaryProblem (XProblem.h:1060-1112):
 * ComputeBoundaryForces, SpreadForce, Interpolate, UpdateBoundaryPosition
 * (XProblem.cpp:8436-8894) over the TImmersedBoundary node list.  Nodes are
 * created once from host arrays and stay on the device:
 *   pos, ref     3 doubles per node (x, y, z; ref = the target-node anchor)
 *   kind         node law (XImmersedBoundary.h / .cpp:654-759), XF_IB_* below
 *   next, prev   neighbour node index or -1 (TNode::neighbors)
 *   dist0        initial distance to next; curv0 3 per node (initialCurvatures)
 *   node_stiff   per-node stiffness (fixed-elastic nodes)
 *   params       {stiffness, stretchingStiffness, bendingStiffness, area}
 * Boxes (velocity, force) are FP64 xf_vec of the staggered grid of `axis`
 * (1 = x, 2 = y, 3 = z); h0 holds the three uniform spacings.  Forces sum in
 * the reference's serial node order (bit-identical); spreading adds markers'
 * contributions with atomics (last-bit order effects). */
enum { XF_IB_ELASTIC = 0, XF_IB_TARGET = 1, XF_IB_FIXED_ELASTIC = 2, XF_IB_PLAIN = 3, XF_IB_FIXED_STRETCHING = 4 };
enum { XF_IB_POS = 0, XF_IB_VEL = 1, XF_IB_FORCE = 2 };   /* fields: 3 * nn doubles each */
typedef struct xf_ib xf_ib;
int xf_ib_create(xf_ctx* ctx, int nn, const double* pos, const double* ref, const int32_t* kind, const int32_t* next,
                 const int32_t* prev, const double* dist0, const double* curv0, const double* node_stiff,
                 const double* params, xf_ib** out);
int xf_ib_destroy(xf_ib* ib);
/* POS: x,y,z per node; VEL and FORCE: the x array, then y, then z (nn each). */
int xf_ib_download(const xf_ib* ib, int field, double* host);
int xf_ib_upload(xf_ib* ib, int field, const double* host);
/* Interpolate (XProblem.cpp:8620-8791): node velocity[axis] from the box. */
int xf_ib_interpolate(xf_ib* ib, const xf_vec* velocity, const double* h0, int axis);
/* UpdateBoundaryPosition (XProblem.cpp:8858-8894): pos[axis] += vel[axis] * tau. */
int xf_ib_update_position(xf_ib* ib, int axis, double tau);
/* ComputeBoundaryForces (XProblem.cpp:8436-8547): force[axis] from positions. */
int xf_ib_compute_forces(xf_ib* ib, int axis);
/* SpreadForce (XProblem.cpp:8550-8617, arithmetic): zero the box, then add
 * every node's force[axis] times its 7^3 cosine-delta weights. */
int xf_ib_spread(xf_ib* ib, xf_vec* force, const double* h0, int axis);

/* ---- learned preconditioner: tensor-core building blocks ------------------ */
/* No counterpart in the reference (it has no learned component).  One
 * 128 x N x K tile on the 5th-generation tensor cores (tcgen05, FP32
 * accumulation in tensor memory): D = A B^T with A 128 x K and B N x K BF16
 * (raw 16-bit patterns, K contiguous), D 128 x N FP32, all host pointers;
 * 16 <= N, K <= 256, multiples of 16.  variant 0 is the operand layout the
 * convolution kernels use; variant 1 swaps the two core-matrix strides of the
 * shared-memory descriptors (a layout check). */
int xf_tc_gemm_bf16(xf_ctx* ctx, int N, int K, const uint16_t* host_a, const uint16_t* host_b, float* host_d,
                    int variant);

/* 3x3x3 convolution of a BF16 activation box on the tensor cores (implicit
 * GEMM: 126- or 128-cell tiles, 27 taps x ci/16 MMAs accumulated in tensor
 * memory).  n1 x n2 x n3 is the level's box (ghost layer included).
 * Activations are stored in channel planes of 8: plane q holds channels
 * 8q .. 8q+7 of every cell, 16 bytes per cell, element (cell c, channel ch) at
 * (ch / 8) * plane_stride + c * 8 + ch % 8 (elements).  `in` points at cell 0
 * of the input slice's first plane (ci channels, plane stride in_ps elements),
 * and every plane extends XF_CONV_MARGIN(n2, n3) cells before cell 0 and after
 * the last cell, all holding 0, as must every ghost and inactive cell (the
 * ghost layer is the zero padding).  weights [27][co][ci] BF16 with tap
 * t = 9 (di+1) + 3 (dj+1) + (dk+1); bias [co] FP32 or NULL; mask [cells] 0/1.
 * out = mask * act(conv + bias), act = ReLU when relu != 0, first out_ch
 * channels: BF16 planes of stride out_pitch elements (out_fp32 = 0, out_ch a
 * multiple of 8) or FP32 cell rows of pitch out_pitch, at `out` (cell 0).
 * ci, co multiples of 16 up to 128; device pointers, 16-byte aligned;
 * asynchronous on the context stream (xf_conv_status reports a tensor-core
 * wait that ran out).  No counterpart in the reference. */
#define XF_CONV_MARGIN(n2, n3) ((int64_t)(n2) * (n3) + (n3) + 1 + 128)
int xf_conv3d_bf16(xf_ctx* ctx, int n1, int n2, int n3, const void* in, int64_t in_ps, int ci, const void* weights,
                   const float* bias, int co, const uint8_t* mask, void* out, int64_t out_pitch, int out_ch,
                   int out_fp32, int relu);
int xf_conv_status(xf_ctx* ctx);

/* The learned preconditioner: a 3-level 3-D U-Net (16/32/64 channels, 3x3x3
 * convolutions on the tensor cores, ReLU, BF16 weights and activations, FP32
 * accumulation, about 0.35 M parameters) over the grid's box; level l+1
 * halves the interior, so the interior dimensions must be multiples of 4.
 * Parameters are one FP32 array, per layer W[27][co][ci] then b[co], layers
 * enc0a (ci padded 1 -> 16), enc0b, enc1a, enc1b, mid_a, mid_b, dec1a (96 in),
 * dec1b, dec0a (48 in), dec0b, out (co padded 1 -> 16; padding forced to 0).
 * No counterpart in the reference. */
typedef struct xf_unet xf_unet;
int xf_unet_create(const xf_grid* g, xf_unet** out);
int xf_unet_destroy(xf_unet* u);
int xf_unet_param_count(const xf_unet* u, int64_t* n);
int xf_unet_set_params(xf_unet* u, const float* host_params);   /* also restarts Adam */
int xf_unet_get_params(xf_unet* u, float* host_params);
int xf_unet_get_grads(xf_unet* u, float* host_grads);
/* z = U-Net(r / rms(r)) on the active cells (FP64 boxes of the grid). */
int xf_unet_apply(xf_unet* u, const xf_vec* r, xf_vec* z);
/* One training step on the pair (r, e), e the error of an iterate and r its
 * residual (A e = r).  With op (the symmetric stencil operator of the grid)
 * the loss is one minus the A-norm cosine of the output z and the error,
 * 1 - (z, r) / sqrt((z, A z) (e, r)), what preconditioned CG convergence
 * depends on; without, the mean over active cells of (z - e / rms e)^2.
 * Writes the loss, accumulates fresh gradients (backward pass: the
 * tensor-core convolution with flipped weights for the input gradients, FP32
 * reductions for the weight gradients) and with apply_update takes an Adam
 * step (lr, beta 0.9 / 0.999). */
int xf_unet_train_step(xf_unet* u, const xf_op* op, const xf_vec* r, const xf_vec* e, double lr, int apply_update,
                       double* loss);
/* Flexible CG, truncated FCG(m): each preconditioned residual is
 * A-orthogonalised against the last m directions (m = opts->reserved[0],
 * 1..8, default 8), robust to a preconditioner that varies between
 * applications.  Preconditioner opts->precond: XF_PRECOND_UNET (u on the
 * operator's grid), XF_PRECOND_UNET2 (u on the coarse grid, see above),
 * XF_PRECOND_JACOBI (Laplace diagonal) or none; FP64, or with
 * XF_PRECOND_UNET2 and opts->precision = XF_PREC_MIXED the correction,
 * residual and directions in FP32 with FP64 dots, refreshed from the true
 * FP64 residual every opts->replace_every iterations or after a 10^3 drop of
 * the FP32 residual (window kept); stops on the true
 * relative residual (opts->rtol).  Plain CG is the fallback (counted in
 * stats->fallbacks): per iteration when z is no descent direction, for good
 * when the residual stalls. */
int xf_solve_fcg(xf_op* op, xf_unet* u, const xf_solve_opts* opts, xf_vec* x, const xf_vec* b,
                 xf_solve_stats* stats);

/* ---- measurement ---------------------------------------------------------- */
/* No counterpart in the reference (a profiling helper).  Times each kernel of
 * one CG iteration on op's grid alone, `reps` launches each, with CUDA events
 * on the context stream, and writes the average ms per launch: [0] FP32
 * stencil q = A p with (p,q), [1] FP32 x/r update with (r,r), [2] FP32
 * direction update, [3] FP64 true residual r32 = b - A x, [4] FP64 stencil,
 * [5] FP32 stencil with the direction update fused in (p' = r + beta p,
 * q = A p', (p', q)) as the solver launches it, or -1 where the grid does not
 * take that path; [6] the same step by the register plane march, else -1;
 * [7] the polynomial preconditioner z = p(A) r with (r, z) (XF_PRECOND_CHEB),
 * or -1; [8] the same launch with the residual update fused in (r' = r -
 * alpha q, e += alpha p', z = p(A) r', (r', r'), (r', z)), or -1; [9] the
 * first pass of the degree-4 preconditioner with the update fused in (r' =
 * r - alpha q, e += alpha p', w = p2(A) r', (r', r')) and [10] its second pass
 * (z = p1(A) w, (r', z)), or -1; [11] a middle pass of a higher degree (w' =
 * p_k(A) w, no dot), or -1; the learned two-level preconditioner's passes
 * on the fine grid (interiors multiples of 4, uniform, no boundary rows, else
 * -1): [12] y = P zc with A y and (y, A y), [13] the smoother's first pass on
 * r - omega A y, [14] its last pass (z = omega y + s p1(A) w, also into the
 * direction slot, with (z, r) and (z, q)).  ms_out holds 15 doubles.  Laplace
 * operators only. */
int xf_profile_cg_kernels(xf_op* op, int reps, double* ms_out);

/* No counterpart in the reference (a self-test).  The time-step passes divide
 * by grid spacings and the time step through their correctly rounded
 * reciprocals and one FMA correction (Markstein's theorem), which must equal
 * the IEEE division bit for bit.  Runs that division and the IEEE one on the
 * device over n hashed operand pairs (mostly in the passes' operand ranges,
 * a quarter fully random bit patterns) and writes the number of pairs whose
 * results differ. */
int xf_selftest_division(xf_ctx* ctx, long long n, unsigned long long seed, long long* mismatches);

/* ---- allocation-free inner product --------------------------------------- */
/* No counterpart in the reference (which has no device memory at all).
 * The masked FP64 dot of xf_dot, sum over c < n with d_mask[c] != 0 (d_mask
 * may be NULL: every element) of d_a[c]*d_b[c], written to *d_out, for
 * callers that cannot allocate device memory: an application that carves all
 * its device memory out of its own pool at start-up (a time loop under a
 * fixed memory budget, or a GPU shared with a library that holds the rest),
 * and loops that must not call cudaFree, which waits for the whole device to
 * go idle.  All pointers are caller-owned
 * device memory; the call is asynchronous on `stream` (a cudaStream_t, NULL
 * for the legacy default stream) and allocates nothing: its scratch is a
 * 64 KiB file-scope device array that every device loading the library keeps
 * until exit.  n beyond XF_NOALLOC_MAX_ELEMS returns XF_ERR_ARG.  Calls share
 * that scratch, so calls that overlap on the GPU race; calls ordered on one
 * stream do not.  The first call on a device resolves the scratch address
 * (cudaGetSymbolAddress, that device current) and keeps it: make that call
 * before any stream capture, and restart the process after a
 * cudaDeviceReset before calling again. */
#define XF_NOALLOC_MAX_ELEMS (8192LL * 256LL * 16LL)
int xf_dot_noalloc(const double* d_a, const double* d_b, const uint8_t* d_mask, int64_t n, double* d_out,
                   void* stream);

#ifdef __cplusplus
}
#endif
#endif /* XFLOW_H */
