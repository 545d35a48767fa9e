/* Test infrastructure only: CPU restatement of the reference algorithms on the
 * pressure-projection path.  Used by tests/ (as the checker), by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline / reference arm.
 * Nothing in the product links this library.
 *
 * Layout: every box is (n1, n2, n3) float64 in C order (k fastest), exactly the
 * reference's double*** [i][j][k] flattened.  Codes are int32 point codes
 * (XMask.h:6-7, XGrid.h:11, XOperator.h:13-18); normals are 3 float64 per cell,
 * all-zero meaning "no normal".  Each routine cites the reference lines it
 * restates; with threads == 1 every loop runs in the reference's order.
 */
#ifndef XF_ORACLE_H
#define XF_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { XFO_OK = 0, XFO_ERR_MASK = 3, XFO_ERR_ARG = 1, XFO_ERR_CHECK = 7 };
enum { XFO_OP_LAPLACE = 0, XFO_OP_VARDIV = 1 };

void xfo_set_threads(int n);
int xfo_get_threads(void);

void xfo_space_mask(const int32_t* codes, int64_t ncell, uint8_t* smask);
int64_t xfo_rn_map(const uint8_t* smask, int n1, int n2, int n3, int32_t* inv_box, int32_t* fwd_ijk);
int xfo_validate(int op, const int32_t* codes, const double* normals, int n1, int n2, int n3, int64_t* bad_cell);

/* y = A x (sign 0), A x + s (sign +1), A x - s (sign -1) on active cells. */
int xfo_apply(int op, const int32_t* codes, const double* normals, const double* hx, const double* hy,
              const double* hz, const double* density, int n1, int n2, int n3, const double* x,
              const double* s, int sign, double* y);

void xfo_lincomb(double p1, const double* s1, double p2, const double* s2, const uint8_t* smask,
                 int64_t ncell, double* z);
double xfo_dot(const double* a, const double* b, const uint8_t* smask, int64_t ncell);
double xfo_norm(const double* a, const uint8_t* smask, int64_t ncell);
double xfo_absmax(const double* a, const uint8_t* smask, const int32_t* inv_box, int64_t ncell, int32_t* rn_index);

typedef struct {
  int iterations;
  double resid;      /* the quantity the stopping rule tested last */
  int status;        /* 0 converged, 13 iteration cap hit */
} xfo_stats;

/* Reference solvers, same arithmetic sequence as XSLAE.cpp; maxit caps the
 * loop (the reference has none), eps as the reference hard-codes when <= 0. */
int xfo_cg_reference(int op, const int32_t* codes, const double* normals, const double* hx,
                     const double* hy, const double* hz, const double* density, int n1, int n2, int n3,
                     const double* x0, const double* b, double eps, int maxit, double* result, xfo_stats* st);
int xfo_bicgstab_reference(int op, const int32_t* codes, const double* normals, const double* hx,
                           const double* hy, const double* hz, const double* density, int n1, int n2,
                           int n3, const double* x0, const double* b, double eps, int maxit, double* result,
                           xfo_stats* st);
int xfo_minres_reference(int op, const int32_t* codes, const double* normals, const double* hx,
                         const double* hy, const double* hz, const double* density, int n1, int n2, int n3,
                         const double* x0, const double* b, double eps, int maxit, double* result,
                         xfo_stats* st);
/* Plain Hestenes-Stiefel CG to ||b - A x||_2 <= rtol ||b||_2 (the FP64 comparison solver). */
int xfo_cg_plain(int op, const int32_t* codes, const double* normals, const double* hx, const double* hy,
                 const double* hz, const double* density, int n1, int n2, int n3, const double* x0,
                 const double* b, double rtol, int maxit, double* result, xfo_stats* st);

void xfo_thomas(int M, double* u, const double* a, const double* b, const double* c, const double* f);

/* Immersed boundary (XProblem.cpp:8436-9046, XImmersedBoundary.cpp:654-759).
 * Nodes: pos/ref 3 per node; kind 0 elastic, 1 target, 2 fixed-elastic,
 * 3 plain, 4 fixed-stretching; next/prev -1 for none. axis 1..3. */
void xfo_ib_interpolate(const double* vel, int n1, int n2, int n3, const double* h0, int axis, int nn,
                        const double* pos, double* node_vel);
void xfo_ib_update(int nn, int axis, double tau, const double* node_vel, double* pos);
void xfo_ib_forces(int nn, int axis, const double* pos, const double* ref, const int32_t* kind,
                   const int32_t* next, const int32_t* prev, const double* dist0, const double* curv0,
                   const double* node_stiff, const double* params, double* force);
void xfo_ib_spread(double* fbox, int n1, int n2, int n3, const double* h0, int axis, int nn, const double* pos,
                   const double* force);

/* Time-step passes of TVPProblem::SolveBySplitting.  Staggered boxes: u is
 * (n1-1) x n2 x n3, v n1 x (n2-1) x n3, w n1 x n2 x (n3-1) for a pressure box
 * n1 x n2 x n3; hxU/hyV/hzW are the separations of the u/v/w grids along their
 * own axis.  density may be NULL (1); border NULL (0).  Return 0, or the
 * reference's throw as XFO_ERR_MASK / XFO_ERR_CHECK with its cell in *bad. */
int xfo_pressure_rhs(const int32_t* codes, int n1, int n2, int n3, const double* u, const double* v,
                     const double* w, const double* hxU, const double* hyV, const double* hzW, const double* density,
                     double tau, const double* border, double* rhs, int64_t* bad);
/* vel box b1 x b2 x b3 with codes; p box one layer longer along axis; hP the
 * pressure separations along axis. */
int xfo_velocity_correct(int axis, const int32_t* codes, int b1, int b2, int b3, const double* prev, const double* p,
                         const double* hP, const double* density, double tau, const double* border, double* cur,
                         int64_t* bad);
double xfo_divergence_max(const int32_t* codes, int n1, int n2, int n3, const double* u, const double* v,
                          const double* w, const double* hxU, const double* hyV, const double* hzW, int32_t* ijk);

/* T1dPackOperator (XOperator.cpp:1135-1350): original (a_*) and transposed
 * (t_*) storages over Rn (0-based rows/cols); arrays of R+1 / 7R entries.
 * Returns nnz or -1. */
int64_t xfo_pack_build(int op, const int32_t* codes, const double* normals, const double* hx, const double* hy,
                       const double* hz, const double* density, int n1, int n2, int n3, int32_t* a_ptr,
                       int32_t* a_cols, double* a_vals, int32_t* t_ptr, int32_t* t_cols, double* t_vals);
void xfo_pack_apply(int64_t R, const int32_t* ptr, const int32_t* cols, const double* vals, const double* x,
                    double* y);
int xfo_bicg_reference(int64_t R, const int32_t* a_ptr, const int32_t* a_cols, const double* a_vals,
                       const int32_t* t_ptr, const int32_t* t_cols, const double* t_vals, const double* b, double eps,
                       int maxit, double* result, xfo_stats* st);

/* Implicit advection-diffusion operator (momentum / transport): y = A x on
 * active cells; the reference's ADI line coefficients summed over the three
 * directions (XProblem.cpp:1236-1238).  flags: 1 convective, 2 diffusive.
 * Dfield (NULL: the constant D) is the per-cell coefficient of the
 * variable-viscosity form (diffCoefVar, XProblem.cpp:3204). */
int xfo_apply_advdiff(const int32_t* codes, const double* normals, const double* hx, const double* hy,
                      const double* hz, const double* u, const double* v, const double* w, double tau, double D,
                      const double* Dfield, int flags, int n1, int n2, int n3, const double* x, double* y);
void xfo_adi_upwind_coeffs(int dir, const int32_t* codes, int n1, int n2, int n3, const double* hx,
                           const double* hy, const double* hz, const double* vecTr, double D, double tau, double* a,
                           double* b, double* c);
void xfo_adi_first_rhs_upwind(const int32_t* codes, int n1, int n2, int n3, const double* hx, const double* hy,
                              const double* hz, const double* f_1, const double* u, const double* v,
                              const double* w, double dc, const double* rp, double tau, double* f);
int xfo_conc_transfer(const int32_t* codes, int n1, int n2, int n3, const double* u, const double* v,
                      const double* w, const double* inlet, double* uTr, double* vTr, double* wTr, double* rpTr,
                      int64_t* bad);

/* Momentum right-hand side of one velocity component (XProblem.cpp:
 * 5088-5419): transfer velocities, face viscosity and rp on the component's
 * b1 x b2 x b3 box (axis 1 u, 2 v, 3 w).  u/v/w are the staggered boxes of the
 * pressure box (b1 + (axis==1)) x (b2 + (axis==2)) x (b3 + (axis==3)), vis
 * that pressure box (NULL: 0), border / force the component box (NULL: 0),
 * normals 3 per component cell (NULL: 0).  XFO_ERR_MASK with the first
 * throwing cell in *bad. */
int xfo_momentum_rhs(int axis, const int32_t* codes, const double* normals, int b1, int b2, int b3,
                     const double* u, const double* v, const double* w, const double* vis, const double* hx,
                     const double* hy, const double* hz, const double* border, const double* force, double* uTr,
                     double* vTr, double* wTr, double* visTr, double* rp, int64_t* bad);

/* The reference's ADI line coefficients (XProblem.cpp:3149-3276): per
 * direction a, b, c at every Actual point, and the first sweep's x-line
 * right-hand side. */
void xfo_adi_line_coeffs(int dir, const int32_t* codes, int n1, int n2, int n3, const double* hx, const double* hy,
                         const double* hz, const double* vecTr, const double* D, double tau, double* a, double* b,
                         double* c);
void xfo_adi_first_rhs(const int32_t* codes, int n1, int n2, int n3, const double* hx, const double* hy,
                       const double* hz, const double* f_1, const double* u, const double* v, const double* w,
                       const double* D, const double* rp, double tau, double* f);

#ifdef __cplusplus
}
#endif

/* VTK legacy ASCII volume (XProblem.cpp:6132-6345) written with the
 * reference's format strings; see xf_oracle.c for the box shapes. */
int xfo_vtk_write(const char* path, int N, int L, int M, const int32_t* node_codes, const double* x, const double* y,
                  const double* z, const double* u, const double* v, const double* w, const int32_t* p_codes,
                  const double* p, const int32_t* d_codes, const double* density, const int32_t* c_codes,
                  const double* conc, const double* vis);
/* "%f\n" of each value (the C library's formatting); returns the length. */
int64_t xfo_format_fixed6(const double* values, int64_t n, char* out, int64_t capacity);
#endif
