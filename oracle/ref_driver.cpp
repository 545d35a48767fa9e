// Test infrastructure only (oracle): a driver that links the reference's own
// compiled classes (XSLAE / XOperator / XSpace / XSpaceModel / XGrid /
// XSeparator / XImmersedBoundary / XProblem) and runs them on inputs written
// by tests/golden/make_golden.py, so that golden vectors come from the
// reference itself rather than from a restatement.
//
// Usage: ref_driver <task> <input.bin> <output.bin>
//   task = matvec | solve | thomas | ib | pack | npy | step | timing
//   (npy writes <output.bin>.npy through the reference's cnpy::npy_save;
//   step runs TVPProblem::SolveBySplitting and writes its VTK files under
//   ../Res/ relative to the working directory, as the reference does)
//
// File format (both directions): a sequence of records
//   char name[32]; char kind ('d' double / 'i' int32); int64 count; data[count]
#include <cstdarg>
#include <ctime>
#include <cstdio>
#include <cstdlib>
#include <unistd.h>
#include <cstring>
#include <cmath>
#include <map>
#include <string>
#include <vector>
#include <stdexcept>

#include "XSLAE.h"
#include "XOperator.h"
#include "XSpace.h"
#include "XSpaceModel.h"
#include "XGrid.h"
#include "XSeparator.h"
#include "XMask.h"
#include "XProblem.h"
#include "XImmersedBoundary.h"
#include "cnpy.h"

#include <omp.h>

struct Rec { char kind; std::vector<double> d; std::vector<int> i; };
typedef std::map<std::string, Rec> Bag;

static Bag read_bag(const char* path) {
  Bag bag;
  FILE* f = fopen(path, "rb");
  if (!f) throw std::runtime_error("cannot open input");
  char name[33];
  while (fread(name, 1, 32, f) == 32) {
    name[32] = 0;
    char kind; long long n;
    if (fread(&kind, 1, 1, f) != 1 || fread(&n, 8, 1, f) != 1) throw std::runtime_error("bad record");
    Rec r; r.kind = kind;
    if (kind == 'd') { r.d.resize(n); if (n && fread(r.d.data(), 8, n, f) != (size_t)n) throw std::runtime_error("short d"); }
    else { r.i.resize(n); if (n && fread(r.i.data(), 4, n, f) != (size_t)n) throw std::runtime_error("short i"); }
    bag[std::string(name)] = r;
  }
  fclose(f);
  return bag;
}

struct Writer {
  FILE* f;
  explicit Writer(const char* p) { f = fopen(p, "wb"); if (!f) throw std::runtime_error("cannot open output"); }
  ~Writer() { fclose(f); }
  void hdr(const char* name, char kind, long long n) {
    char b[32]; memset(b, 0, 32); strncpy(b, name, 31);
    fwrite(b, 1, 32, f); fwrite(&kind, 1, 1, f); fwrite(&n, 8, 1, f);
  }
  void d(const char* name, const std::vector<double>& v) { hdr(name, 'd', v.size()); if (!v.empty()) fwrite(v.data(), 8, v.size(), f); }
  void i(const char* name, const std::vector<int>& v) { hdr(name, 'i', v.size()); if (!v.empty()) fwrite(v.data(), 4, v.size(), f); }
  void s(const char* name, double x) { d(name, std::vector<double>(1, x)); }
  void n(const char* name, int x) { i(name, std::vector<int>(1, x)); }
};

static const std::vector<double>& D(Bag& b, const char* k) {
  Bag::iterator it = b.find(k);
  if (it == b.end()) { fprintf(stderr, "missing %s\n", k); throw std::runtime_error("missing record"); }
  return it->second.d;
}
static const std::vector<int>& I(Bag& b, const char* k) {
  Bag::iterator it = b.find(k);
  if (it == b.end()) { fprintf(stderr, "missing %s\n", k); throw std::runtime_error("missing record"); }
  return it->second.i;
}

// ---------------------------------------------------------------------------
// Grid + space model exactly as XProblem.cpp:3989-4049 (BuildLocalGrid) and
// XProblem.cpp:4116-4207 (LocalPrepareVariables) build them.
struct Setup {
  int n1, n2, n3;
  T3dNormalGrid* grid;
  int model;
  std::vector<double> hx, hy, hz;
};

static Setup build(Bag& b, int modelName) {
  Setup s;
  const std::vector<int>& dims = I(b, "dims");
  s.n1 = dims[0]; s.n2 = dims[1]; s.n3 = dims[2];
  const std::vector<double>& X = D(b, "x_nodes");
  const std::vector<double>& Y = D(b, "y_nodes");
  const std::vector<double>& Z = D(b, "z_nodes");
  TSeparator* sep1 = new TRandomSeparator(s.n1, X.data());
  TSeparator* sep2 = new TRandomSeparator(s.n2, Y.data());
  TSeparator* sep3 = new TRandomSeparator(s.n3, Z.data());
  const std::vector<int>& codes = I(b, "codes");
  const std::vector<double>& nrm = D(b, "normals");
  T3dNumberMask& mask = *(new T3dNumberMask(s.n1, s.n2, s.n3));
  T3dVector**** normals = new T3dVector***[s.n1];
  for (int i = 0; i < s.n1; i++) {
    normals[i] = new T3dVector**[s.n2];
    for (int j = 0; j < s.n2; j++) {
      normals[i][j] = new T3dVector*[s.n3];
      for (int k = 0; k < s.n3; k++) {
        size_t c = ((size_t)i * s.n2 + j) * s.n3 + k;
        mask[i][j][k] = codes[c];
        T3dVector* nv = NULL;
        if (nrm[3 * c] != 0 || nrm[3 * c + 1] != 0 || nrm[3 * c + 2] != 0) {
          nv = new T3dVector; nv->X = nrm[3 * c]; nv->Y = nrm[3 * c + 1]; nv->Z = nrm[3 * c + 2];
        }
        normals[i][j][k] = nv;
      }
    }
  }
  s.grid = new T3dNormalGrid(sep1, sep2, sep3, mask, normals);
  for (int q = 0; q < s.n1 - 1; q++) s.hx.push_back(s.grid->GetSeparator1().Separation[q]);
  for (int q = 0; q < s.n2 - 1; q++) s.hy.push_back(s.grid->GetSeparator2().Separation[q]);
  for (int q = 0; q < s.n3 - 1; q++) s.hz.push_back(s.grid->GetSeparator3().Separation[q]);

  // Space mask: grid codes -> {0,1} as XProblem.cpp:4155-4182.
  T3dNumberMask& spaceMask = s.grid->GetMask().Copy();
  for (int i = 0; i < s.n1; i++)
    for (int j = 0; j < s.n2; j++)
      for (int k = 0; k < s.n3; k++) {
        int m = spaceMask[i][j][k];
        if (m == TActualPoint || m == TFictivePoint) spaceMask[i][j][k] = m;
        else if (m == TDefinedBorderPoint || m == TEquationBorderPoint) spaceMask[i][j][k] = TFictivePoint;
        else spaceMask[i][j][k] = TActualPoint;
      }
  TMask** masks = new TMask*[1];
  masks[0] = &spaceMask;
  TRnRelease3dSpaceModel* model = new TRnRelease3dSpaceModel(1, masks);
  TRnSpace::AddModel(modelName, model, false);
  s.model = modelName;
  return s;
}

static TRnRelease3dSpace& vec_from(Setup& s, const std::vector<double>& v) {
  TRnRelease3dSpace& x = *(new TRnRelease3dSpace(s.model));
  for (int i = 0; i < s.n1; i++)
    for (int j = 0; j < s.n2; j++)
      for (int k = 0; k < s.n3; k++) x[i][j][k] = v[((size_t)i * s.n2 + j) * s.n3 + k];
  return x;
}
static std::vector<double> vec_to(Setup& s, TRnRelease3dSpace& x) {
  std::vector<double> v((size_t)s.n1 * s.n2 * s.n3);
  for (int i = 0; i < s.n1; i++)
    for (int j = 0; j < s.n2; j++)
      for (int k = 0; k < s.n3; k++) v[((size_t)i * s.n2 + j) * s.n3 + k] = x[i][j][k];
  return v;
}

// ---------------------------------------------------------------------------
static void task_matvec(Bag& b, Writer& w) {
  Setup s = build(b, 11);
  w.d("hx", s.hx); w.d("hy", s.hy); w.d("hz", s.hz);
  TRnRelease3dSpace& x = vec_from(s, D(b, "x"));
  TRnRelease3dSpace& sv = vec_from(s, D(b, "s"));
  TRnRelease3dSpace& rho = vec_from(s, D(b, "density"));
  TNodesGrid** grids = new TNodesGrid*[1]; grids[0] = s.grid;
  T3dLaplaceOperator& A = *(new T3dLaplaceOperator(s.model, 1, grids));
  T3dVariableDivergentedOperator& V = *(new T3dVariableDivergentedOperator(s.model, 1, grids));
  V.withDensity(rho);
  const std::vector<double>& yinit = D(b, "y_init");

  // a6 / a10: y |= A(x), A(x)+s, A(x)-s (inactive cells keep y_init)
  { TRnRelease3dSpace& y = vec_from(s, yinit); y |= ((TRnLinearOperator&)A)(x); w.d("lap_y", vec_to(s, y)); delete &y; }
  { TRnRelease3dSpace& y = vec_from(s, yinit); y |= ((TRnLinearOperator&)A)(x) + sv; w.d("lap_y_plus", vec_to(s, y)); delete &y; }
  { TRnRelease3dSpace& y = vec_from(s, yinit); y |= ((TRnLinearOperator&)A)(x) - sv; w.d("lap_y_minus", vec_to(s, y)); delete &y; }
  // a7
  // (only on grids whose PreNormal rows lie off the box faces: on the faces
  // the reference's PreNormal branch reads outside its separation and density
  // arrays, XOperator.cpp:2104-2130, 2211-2213)
  if (b.count("vardiv")) { TRnRelease3dSpace& y = vec_from(s, yinit); y |= ((TRnLinearOperator&)V)(x); w.d("vd_y", vec_to(s, y)); delete &y; }
  // a11: masked linear combinations
  double p1 = D(b, "p1")[0], p2 = D(b, "p2")[0];
  { TRnRelease3dSpace& z = vec_from(s, yinit); z |= p1 * x + p2 * sv; w.d("lc_p1x_p2s", vec_to(s, z)); delete &z; }
  { TRnRelease3dSpace& z = vec_from(s, yinit); z |= x - sv; w.d("lc_x_minus_s", vec_to(s, z)); delete &z; }
  { TRnRelease3dSpace& z = vec_from(s, yinit); z |= x + p2 * sv; w.d("lc_x_p2s", vec_to(s, z)); delete &z; }
  { TRnRelease3dSpace& z = vec_from(s, yinit); z |= p1 * x; w.d("lc_p1x", vec_to(s, z)); delete &z; }
  { TRnRelease3dSpace& z = vec_from(s, yinit); z |= 0; w.d("lc_zero", vec_to(s, z)); delete &z; }
  { TRnRelease3dSpace& z = vec_from(s, yinit); z.Assign(x); w.d("assign_x", vec_to(s, z)); delete &z; }
  // a12: reductions
  w.s("dot_xs", (x, sv));
  w.s("norm_x", x.Norma(0));
  w.s("dot_x_As", (x, ((TRnLinearOperator&)A)(sv)));
  { int idx = -7; double m = x.GetAbsMaxElement(idx); w.s("absmax_x", m); w.n("absmax_x_index", idx); }
  { int idx = -7; double m = sv.GetAbsMaxElement(idx); w.s("absmax_s", m); w.n("absmax_s_index", idx); }
  { int idx = -7; double m = x.GetAbsMinElement(idx); w.s("absmin_x", m); w.n("absmin_x_index", idx); }
  // a14: Rn numbering
  int R = x.EndIndex;
  w.n("end_index", R);
  std::vector<int> fwd; fwd.reserve(3 * R);
  std::vector<double> rn_vals; rn_vals.reserve(R);
  for (int rn = 1; rn <= R; rn++) rn_vals.push_back(((TRnSpace&)x)[rn]);
  w.d("x_by_rn", rn_vals);
  delete &V; delete &A; delete &x; delete &sv; delete &rho;
}

// ---------------------------------------------------------------------------
// Krylov solves through the reference TSLAE (XSLAE.cpp). op = 0 Laplace,
// 1 variable-density; method = 0 CG, 1 BiCGStab, 2 MinRes.
static void task_solve(Bag& b, Writer& w) {
  Setup s = build(b, 21);
  TNodesGrid** grids = new TNodesGrid*[1]; grids[0] = s.grid;
  int op = I(b, "op")[0], method = I(b, "method")[0];
  TRnRelease3dSpace& x = vec_from(s, D(b, "x0"));
  TRnRelease3dSpace& rhs = vec_from(s, D(b, "b"));
  T3dLaplaceOperator* A;
  if (op == 0) A = new T3dLaplaceOperator(s.model, 1, grids);
  else {
    T3dVariableDivergentedOperator* V = new T3dVariableDivergentedOperator(s.model, 1, grids);
    TRnRelease3dSpace& rho = vec_from(s, D(b, "density"));
    V->withDensity(rho);
    A = V;
  }
  TSLAE* slae = new TSLAE(*A, x, rhs);
  if (method == 0) slae->SolveByConjugateGradients();
  else if (method == 1) slae->SolveByBiConjugateGradientsStab();
  else slae->SolveByMinimalResiduals();
  TRnRelease3dSpace& res = dynamic_cast<TRnRelease3dSpace&>(const_cast<TRnSpace&>((const TRnSpace&)slae->Result));
  w.d("result", vec_to(s, res));
  // The residual the reference's own stopping rule sees, recomputed here.
  TRnRelease3dSpace& r = *(new TRnRelease3dSpace(s.model));
  r |= ((TRnLinearOperator&)*A)(res) - rhs;
  w.s("resid_l2", r.Norma(0));
  w.s("resid_inf", r.GetAbsMaxElement());
}

// ---------------------------------------------------------------------------
// a8/a9/a2: T1dPackOperator built from the Laplace operator exactly as
// XProblem.cpp:700-760 does (Rn space model of all-Actual points, NULL
// transform vector), its row and column storages, A x and A^T x on a seeded x,
// and TSLAE::SolveByBiConjugateGradients on the packed system.
class PackProbe : public T1dPackOperator {
 public:
  PackProbe(int model, const TRnLinearOperator& A, double** v)
      : TRnLinearOperator(model), T1dPackOperator(model, A, v) {}  // virtual base first
  void dump(Writer& w, bool transpose) {
    int n = transpose ? fRowsCountT : fRowsCount;
    int* cnt = transpose ? fRowsElementsCountT : fRowsElementsCount;
    double** m = transpose ? fMatrixPackT : fMatrixPack;
    int** c = transpose ? fColumnsT : fColumns;
    std::vector<int> ptr(1, 0), cols;
    std::vector<double> vals;
    for (int r = 0; r < n; r++) {
      for (int q = 0; q < cnt[r]; q++) { cols.push_back(c[r][q]); vals.push_back(m[r][q]); }
      ptr.push_back((int)cols.size());
    }
    w.i(transpose ? "t_ptr" : "a_ptr", ptr);
    w.i(transpose ? "t_cols" : "a_cols", cols);
    w.d(transpose ? "t_vals" : "a_vals", vals);
  }
};

static void task_pack(Bag& b, Writer& w) {
  Setup s = build(b, 31);
  TNodesGrid** grids = new TNodesGrid*[1]; grids[0] = s.grid;
  T3dLaplaceOperator& A = *(new T3dLaplaceOperator(s.model, 1, grids));
  TRnRelease3dSpace& probe = vec_from(s, D(b, "x"));
  int RN = probe.EndIndex;
  T1dNumberMask& maskRn = *(new T1dNumberMask(RN));
  for (int rn = 0; rn < RN; rn++) maskRn[rn] = TActualPoint;
  TMask** masksRn = new TMask*[1];
  masksRn[0] = &maskRn;
  TRnRelease1dSpaceModel& modelRn = *(new TRnRelease1dSpaceModel(1, masksRn));
  const int nameRn = 777;
  TRnSpace::AddModel(nameRn, &modelRn, false);
  double* nullVector = NULL;
  PackProbe& P = *(new PackProbe(nameRn, A, &nullVector));
  P.dump(w, false);
  P.dump(w, true);
  TRnRelease1dSpace& x = *(new TRnRelease1dSpace(nameRn));
  TRnRelease1dSpace& y = *(new TRnRelease1dSpace(nameRn));
  const std::vector<double>& xr = D(b, "x_rn");
  for (int rn = 0; rn < RN; rn++) x[rn] = xr[rn];
  y |= ((TRnLinearOperator&)P)(x);
  std::vector<double> out(RN);
  for (int rn = 0; rn < RN; rn++) out[rn] = y[rn];
  w.d("ax", out);
  ~P;
  y |= ((TRnLinearOperator&)P)(x);
  for (int rn = 0; rn < RN; rn++) out[rn] = y[rn];
  w.d("atx", out);
  ~P;
  if (b.count("b_rn")) {
    TRnRelease1dSpace& rhs = *(new TRnRelease1dSpace(nameRn));
    TRnRelease1dSpace& x0 = *(new TRnRelease1dSpace(nameRn));
    const std::vector<double>& br = D(b, "b_rn");
    for (int rn = 0; rn < RN; rn++) { rhs[rn] = br[rn]; x0[rn] = 0; }
    TSLAE* slae = new TSLAE(P, x0, rhs);
    slae->SolveByBiConjugateGradients();
    TRnRelease1dSpace& res = dynamic_cast<TRnRelease1dSpace&>(const_cast<TRnSpace&>((const TRnSpace&)slae->Result));
    for (int rn = 0; rn < RN; rn++) out[rn] = res[rn];
    w.d("bicg_x", out);
  }
}

// ---------------------------------------------------------------------------
// a5: TSLAE::SolveByScalarRunning on a batch of lines.
static void task_thomas(Bag& b, Writer& w) {
  int nl = I(b, "nlines")[0], M = I(b, "M")[0];
  std::vector<double> u = D(b, "u");
  const std::vector<double>& a = D(b, "a"), &bb = D(b, "b"), &c = D(b, "c"), &f = D(b, "f");
  for (int l = 0; l < nl; l++) {
    size_t o = (size_t)l * (M + 1);
    TSLAE::SolveByScalarRunning(M, &u[o], &a[o], &bb[o], &c[o], &f[o]);
  }
  w.d("u", u);
}

// ---------------------------------------------------------------------------
// a17-a19: the reference's IB driver methods, reached through a subclass that
// only widens access.  No Initialize(): the boundary is assembled here.
class IBProbe : public TImmersedBoundaryProblem {
 public:
  IBProbe(double tEnd, double tau) : TImmersedBoundaryProblem(tEnd, tau, 100.0, 1.0) {
    fTimeSeparator = new TUniformSeparator(0, tEnd, tau);  // as THydrodynamicsProblem::Initialize
  }
  double step() { return fTimeSeparator->SeparationValue; }
  virtual TMaskGenerator* CreateStatement() { return NULL; }
  void setBoundary(TImmersedBoundary* bnd) { fBoundary = bnd; }
  void interp(TRnRelease3dSpace& v, T3dNormalGrid* g, int axis) { Interpolate(v, g, axis, 1); }
  void update(int axis) { UpdateBoundaryPosition(axis, 1); }
  void forces(int axis) { ComputeBoundaryForces(axis, 1); }
  void spread(TRnRelease3dSpace& f, T3dNormalGrid& gc, T3dNormalGrid* g, int axis) { SpreadForce(f, gc, g, axis, 1); }
  ~IBProbe() {}
};

class ProbeBoundary : public TImmersedBoundary {
 public:
  double area;
  double GetArea() { return area; }
  double GetYCenter() { return 0; }
  double GetZCenter() { return 0; }
};

static void task_ib(Bag& b, Writer& w) {
  Setup s = build(b, 31);
  double tau = D(b, "tau")[0];
  IBProbe* P = new IBProbe(1000 * tau, tau);
  const std::vector<double>& pos = D(b, "pos");      // 3*n
  const std::vector<double>& ref = D(b, "ref");      // 3*n
  const std::vector<int>& kind = I(b, "kind");       // 0 elastic, 1 target, 2 fixed-elastic, 3 plain
  const std::vector<int>& nxt = I(b, "next");        // -1 none
  const std::vector<int>& prv = I(b, "prev");
  const std::vector<double>& d0 = D(b, "dist0");
  const std::vector<double>& curv0 = D(b, "curv0");  // 3*n
  const std::vector<double>& kst = D(b, "node_stiff");
  const std::vector<double>& prm = D(b, "params");   // stiffness, stretching, bending, area
  int n = (int)kind.size();
  ProbeBoundary* B = new ProbeBoundary();
  B->stiffness = prm[0]; B->stretchingStiffness = prm[1]; B->bendingStiffness = prm[2]; B->area = prm[3];
  B->nodesCount = n;
  B->nodes = new TNode*[n];
  for (int q = 0; q < n; q++) {
    TNode* nd;
    if (kind[q] == 0) nd = new TElasticNode();
    else if (kind[q] == 1) nd = new TTargetNode();
    else if (kind[q] == 2) nd = new TFixedElasticNode();
    else nd = new TNode();
    nd->x = pos[3 * q]; nd->y = pos[3 * q + 1]; nd->z = pos[3 * q + 2];
    nd->xRef = ref[3 * q]; nd->yRef = ref[3 * q + 1]; nd->zRef = ref[3 * q + 2];
    nd->TNode::type = ELASTIC_NODE;  // never FIXED here: the mask side effect is not part of the arithmetic
    nd->stretchingStiffness = kst[q];
    nd->boundary = B;
    nd->neighbors.initialDistanceNext = d0[q];
    nd->neighbors.initialCurvatures[OX] = curv0[3 * q];
    nd->neighbors.initialCurvatures[OY] = curv0[3 * q + 1];
    nd->neighbors.initialCurvatures[OZ] = curv0[3 * q + 2];
    B->nodes[q] = nd;
  }
  for (int q = 0; q < n; q++) {
    B->nodes[q]->neighbors.next = nxt[q] >= 0 ? B->nodes[nxt[q]] : NULL;
    B->nodes[q]->neighbors.prev = prv[q] >= 0 ? B->nodes[prv[q]] : NULL;
  }
  P->setBoundary(B);
  w.s("tau_eff", P->step());
  TRnRelease3dSpace& vel = vec_from(s, D(b, "velocity"));
  int axis = I(b, "axis")[0];
  // GetForce order (XProblem.cpp:8350-8353): interpolate, move, forces, spread.
  P->interp(vel, s.grid, axis);
  std::vector<double> vout(n);
  for (int q = 0; q < n; q++) vout[q] = axis == 1 ? B->nodes[q]->xVel : axis == 2 ? B->nodes[q]->yVel : B->nodes[q]->zVel;
  w.d("node_vel", vout);
  P->update(axis);
  std::vector<double> pout(3 * n);
  for (int q = 0; q < n; q++) { pout[3 * q] = B->nodes[q]->x; pout[3 * q + 1] = B->nodes[q]->y; pout[3 * q + 2] = B->nodes[q]->z; }
  w.d("pos_after", pout);
  P->forces(axis);
  std::vector<double> fout(n);
  for (int q = 0; q < n; q++) fout[q] = axis == 1 ? B->nodes[q]->xForce : axis == 2 ? B->nodes[q]->yForce : B->nodes[q]->zForce;
  w.d("node_force", fout);
  TRnRelease3dSpace& force = *(new TRnRelease3dSpace(s.model));
  P->spread(force, *s.grid, s.grid, axis);
  w.d("force_box", vec_to(s, force));
}

// cnpy::npy_save (cnpy.h:66-112) of "data" with shape "shape", as the time
// loop's NPY output calls it (XProblem.cpp:6545-6590).
static void task_npy(Bag& b, const char* out) {
  const std::vector<int>& sh = b["shape"].i;
  std::vector<unsigned int> shape(sh.begin(), sh.end());
  cnpy::npy_save(std::string(out) + ".npy", b["data"].d.data(), shape.data(), (unsigned int)shape.size(), "w");
}

// ---------------------------------------------------------------------------
// The time step itself: TVPProblem::SolveBySplitting (XProblem.cpp:4255-6650)
// run for two steps on grids, border values, forces and an initial
// concentration taken from the input, through a subclass that supplies them
// by the reference's own virtual hooks (BuildGrid*, GetBorderCondition*,
// GetForce, InitialConcentrationDistribution) and reads state back through
// others (GetForce's transfer-velocity argument, ComputeStress,
// CountBoundaryP/Concentration/Viscosity).  Three routines the step calls
// from XSLAE.o and the C library are wrapped at link time
// (-Wl,--wrap, oracle/Makefile) so that values that live only inside
// SolveBySplitting can be read as they pass:
//   TSLAE::SolveByBiConjugateGradientsStab  the pressure system's right-hand
//       side and warm start (XProblem.cpp:5570-5588); with zero_p set, the
//       capture step's solve is replaced by p = 0, so that the velocity
//       correction (XProblem.cpp:5663, u = u_ - tau gradP / rho) hands back
//       the intermediate velocity u_ itself;
//   TSLAE::SolveByScalarRunning  every ADI line system (a, b, c, f and the
//       solution) of the capture step, in call order;
//   __printf_chk  the control balance's value and cell (XProblem.cpp:5829),
//       read from the call's arguments rather than from the printed text.
// Nothing else is replaced: the rest of the step is the reference's code.
static Writer* g_out = NULL;
static int g_step = 0;          // time step in progress (from the hooks' arguments)
static int g_capture = 2;       // the step whose values are written
static int g_zero_p = 0;
static std::vector<int> g_line_m, g_line_eq;
static std::vector<double> g_line_a, g_line_b, g_line_c, g_line_f, g_line_u;

struct SlaePeek : TSLAE {   // pointers to TSLAE's protected members (no object of this type exists)
  static TRnSpace* TSLAE::*fx_() { return &SlaePeek::fx; }
  static TRnSpace* TSLAE::*fb_() { return &SlaePeek::fb; }
  static TRnSpace* TSLAE::*fres_() { return &SlaePeek::fResult; }
};

static std::vector<double> box_of(TRnSpace& v, int n1, int n2, int n3) {
  TRnRelease3dSpace& x = dynamic_cast<TRnRelease3dSpace&>(v);
  std::vector<double> out((size_t)n1 * n2 * n3);
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) out[((size_t)i * n2 + j) * n3 + k] = x[i][j][k];
  return out;
}
static std::vector<int> g_pdims;   // pressure box

extern "C" void __real__ZN5TSLAE31SolveByBiConjugateGradientsStabEv(TSLAE* self);
extern "C" void __wrap__ZN5TSLAE31SolveByBiConjugateGradientsStabEv(TSLAE* self) {
  const bool cap = g_out && g_step == g_capture;
  if (cap) {
    g_out->d("rhs", box_of(*(self->*SlaePeek::fb_()), g_pdims[0], g_pdims[1], g_pdims[2]));
    g_out->d("p0", box_of(*(self->*SlaePeek::fx_()), g_pdims[0], g_pdims[1], g_pdims[2]));
  }
  if (cap && g_zero_p) {
    *(self->*SlaePeek::fres_()) |= 0;
    return;
  }
  __real__ZN5TSLAE31SolveByBiConjugateGradientsStabEv(self);
}

extern "C" void __real__ZN5TSLAE20SolveByScalarRunningEiPdPKdS2_S2_S2_(int, double*, const double*, const double*,
                                                                         const double*, const double*);
extern "C" void __wrap__ZN5TSLAE20SolveByScalarRunningEiPdPKdS2_S2_S2_(int M, double* U, const double* A,
                                                                         const double* B, const double* C,
                                                                         const double* F) {
  __real__ZN5TSLAE20SolveByScalarRunningEiPdPKdS2_S2_S2_(M, U, A, B, C, F);
  if (!(g_out && g_step == g_capture)) return;
  g_line_m.push_back(M);
  g_line_eq.push_back(omp_get_thread_num());
  g_line_a.insert(g_line_a.end(), A, A + M + 1);
  g_line_b.insert(g_line_b.end(), B, B + M + 1);
  g_line_c.insert(g_line_c.end(), C, C + M + 1);
  g_line_f.insert(g_line_f.end(), F, F + M + 1);
  g_line_u.insert(g_line_u.end(), U, U + M + 1);
}

// SolveBySplitting's teardown (XProblem.cpp:6652-6680) deletes the pressure
// vector, the right-hand side and the operator twice: once through
// `delete slae` (TSLAE::~TSLAE deletes its A, x and b, XSLAE.cpp:21-30) and
// again by name.  Every value has been read by then, so the step task writes
// its last records and ends the process when that teardown announces itself.
static void step_finish() {
  g_out->i("line_m", g_line_m);
  g_out->i("line_thread", g_line_eq);
  g_out->d("line_a", g_line_a);
  g_out->d("line_b", g_line_b);
  g_out->d("line_c", g_line_c);
  g_out->d("line_f", g_line_f);
  g_out->d("line_u", g_line_u);
  fclose(g_out->f);
  fflush(stderr);
  _exit(0);
}
extern "C" int __wrap___printf_chk(int flag, const char* fmt, ...) {
  (void)flag;
  if (g_out && strncmp(fmt, "Deleting temporary objects: Starting", 36) == 0) step_finish();
  va_list ap;
  va_start(ap, fmt);
  if (g_out && g_step == g_capture && strncmp(fmt, "Control balance: OK. (point", 27) == 0) {
    va_list aq;
    va_copy(aq, ap);
    int i = va_arg(aq, int), j = va_arg(aq, int), k = va_arg(aq, int);
    double v = va_arg(aq, double);
    va_end(aq);
    std::vector<int> ijk(3);
    ijk[0] = i; ijk[1] = j; ijk[2] = k;
    g_out->i("div_ijk", ijk);
    g_out->s("div_max", v);
  }
  int r = vfprintf(stderr, fmt, ap);   // the reference's progress log, kept off the driver's stdout
  va_end(ap);
  return r;
}

static T3dNormalGrid* grid_from(Bag& b, const std::string& pre) {
  const std::vector<int>& dims = I(b, (pre + "_dims").c_str());
  const int n1 = dims[0], n2 = dims[1], n3 = dims[2];
  TSeparator* s1 = new TRandomSeparator(n1, D(b, (pre + "_x").c_str()).data());
  TSeparator* s2 = new TRandomSeparator(n2, D(b, (pre + "_y").c_str()).data());
  TSeparator* s3 = new TRandomSeparator(n3, D(b, (pre + "_z").c_str()).data());
  const std::vector<int>& codes = I(b, (pre + "_codes").c_str());
  const std::vector<double>* nrm = b.count(pre + "_nrm") ? &D(b, (pre + "_nrm").c_str()) : NULL;
  T3dNumberMask& mask = *(new T3dNumberMask(n1, n2, n3));
  T3dVector**** normals = new T3dVector***[n1];
  for (int i = 0; i < n1; i++) {
    normals[i] = new T3dVector**[n2];
    for (int j = 0; j < n2; j++) {
      normals[i][j] = new T3dVector*[n3];
      for (int k = 0; k < n3; k++) {
        const size_t c = ((size_t)i * n2 + j) * n3 + k;
        mask[i][j][k] = codes[c];
        T3dVector* nv = NULL;
        if (nrm && ((*nrm)[3 * c] != 0 || (*nrm)[3 * c + 1] != 0 || (*nrm)[3 * c + 2] != 0)) {
          nv = new T3dVector; nv->X = (*nrm)[3 * c]; nv->Y = (*nrm)[3 * c + 1]; nv->Z = (*nrm)[3 * c + 2];
        }
        normals[i][j][k] = nv;
      }
    }
  }
  return new T3dNormalGrid(s1, s2, s3, mask, normals);
}

class StepProblem : public TVPProblem {
 public:
  StepProblem(Bag& bag, double tEnd, double tau, double mu1, double mu2, double rho1, double rho2)
      : TVPProblem(tEnd, tau, mu1, mu2, rho1, rho2), b(bag) {}
  void run() {
    Initialize();
    Solve();
  }
  using TVPProblem::ComputeStress;

 protected:
  Bag& b;
  double box_value(const char* pre, const char* rec, int i, int j, int k) {
    const std::vector<int>& dims = I(b, (std::string(pre) + "_dims").c_str());
    return D(b, rec)[((size_t)i * dims[1] + j) * dims[2] + k];
  }
  std::vector<int> dims(const char* pre) { return I(b, (std::string(pre) + "_dims").c_str()); }
  void record(const char* name, TRnSpace& v, const char* pre) {
    std::vector<int> d = dims(pre);
    g_out->d(name, box_of(v, d[0], d[1], d[2]));
  }
  virtual TMaskGenerator* CreateStatement() { return NULL; }
  virtual TNodesGrid* BuildGrid() { return grid_from(b, "n"); }
  virtual TNodesGrid* BuildGridU() { return grid_from(b, "u"); }
  virtual TNodesGrid* BuildGridV() { return grid_from(b, "v"); }
  virtual TNodesGrid* BuildGridW() { return grid_from(b, "w"); }
  virtual TNodesGrid* BuildGridP() { return grid_from(b, "p"); }
  virtual double GetBorderConditionU(int i, int j, int k, int) { return box_value("u", "u_bc", i, j, k); }
  virtual double GetBorderConditionV(int i, int j, int k, int) { return box_value("v", "v_bc", i, j, k); }
  virtual double GetBorderConditionW(int i, int j, int k, int) { return box_value("w", "w_bc", i, j, k); }
  virtual double GetBorderConditionP(int i, int j, int k, int) { return box_value("p", "p_bc", i, j, k); }
  virtual bool InitialConcentrationDistribution(int i, int j, int k, int, int, int) {
    return box_value("p", "conc0", i, j, k) != 0;
  }
  virtual void GetForce(TRnRelease3dSpace& force, T3dNormalGrid&, T3dNormalGrid&, TRnRelease3dSpace& velocity,
                        const int axis, const int ts) {
    g_step = ts;
    const char* pre = axis == 1 ? "u" : axis == 2 ? "v" : "w";
    if (ts == g_capture) record(axis == 1 ? "tr_1" : axis == 2 ? "tr_2" : "tr_3", velocity, pre);
    std::vector<int> d = dims(pre);
    const std::vector<double>& f = D(b, axis == 1 ? "force_u" : axis == 2 ? "force_v" : "force_w");
    for (int i = 0; i < d[0]; i++)
      for (int j = 0; j < d[1]; j++)
        for (int k = 0; k < d[2]; k++) force[i][j][k] = f[((size_t)i * d[1] + j) * d[2] + k];
  }
  virtual void ComputeStress(TRnRelease3dSpace& U, TRnRelease3dSpace& V, TRnRelease3dSpace& W, int ts) {
    g_step = ts;
    const char* nu = ts == g_capture ? "u" : "s1_u";
    const char* nv = ts == g_capture ? "v" : "s1_v";
    const char* nw = ts == g_capture ? "w" : "s1_w";
    if (ts == g_capture || ts == g_capture - 1) {
      record(nu, U, "u");
      record(nv, V, "v");
      record(nw, W, "w");
    }
  }
  virtual void CountBoundaryP(TRnRelease3dSpace& p) {
    if (g_step == g_capture) record("p", p, "p");
    else if (g_step == g_capture - 1) record("s1_p", p, "p");
  }
  virtual void CountBoundaryConcentration(TRnRelease3dSpace& c) {
    if (g_step == g_capture) record("cnc", c, "p");
    else if (g_step == g_capture - 1) record("s1_cnc", c, "p");
  }
  virtual void CountBoundaryViscosity(TRnRelease3dSpace& v) {
    if (g_step == g_capture) record("vis", v, "p");
    else if (g_step == g_capture - 1) record("s1_vis", v, "p");
  }
};

static void task_step(Bag& b, Writer& w) {
  const std::vector<double>& prm = D(b, "params");   // tau, mu1, mu2, rho1, rho2
  g_out = &w;
  g_pdims = I(b, "p_dims");
  g_capture = 2;
  g_zero_p = I(b, "zero_p")[0];
  TProblem::GlobalUsePackOperator = false;   // the TSLAE-on-the-box path (XFlow.cpp:51)
  TProblem::GlobalTurbulenceMode = false;
  TProblem::GlobalSaveStep = 2;              // VTK of steps 1 and 2
  StepProblem* P = new StepProblem(b, 2 * prm[0], prm[0], prm[1], prm[2], prm[3], prm[4]);
  P->run();   // ends in step_finish() at the reference's teardown
  throw std::runtime_error("the time step returned without reaching its teardown");
}

// ---------------------------------------------------------------------------
// Timing of the reference's own vector and operator calls, to anchor the
// oracle port's CPU times: `reps` of y |= A(x) (XSpace.cpp:3013-3217 driving
// XOperator.cpp:938-1129), (x, y) (XSpace.cpp:3261-3342) and
// z |= p1 x + p2 y (XSpace.cpp:2489-3010), each averaged, then (when "cg" is
// given) one TSLAE::SolveByConjugateGradients from x0 (XSLAE.cpp:56-157,
// its own absolute 1e-5 stop rule) timed whole.
static double now_s() {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec + 1e-9 * t.tv_nsec;
}

static void task_timing(Bag& b, Writer& w) {
  Setup s = build(b, 31);
  const int reps = I(b, "reps")[0];
  TNodesGrid** grids = new TNodesGrid*[1]; grids[0] = s.grid;
  T3dLaplaceOperator& A = *(new T3dLaplaceOperator(s.model, 1, grids));
  TRnRelease3dSpace& x = vec_from(s, D(b, "x"));
  TRnRelease3dSpace& y = vec_from(s, D(b, "x"));
  TRnRelease3dSpace& z = vec_from(s, D(b, "x"));
  double t0 = now_s();
  for (int q = 0; q < reps; q++) y |= ((TRnLinearOperator&)A)(x);
  w.s("matvec_s", (now_s() - t0) / reps);
  double acc = 0;
  t0 = now_s();
  for (int q = 0; q < reps; q++) acc += (x, y);
  w.s("dot_s", (now_s() - t0) / reps);
  w.s("dot_sum", acc);
  t0 = now_s();
  for (int q = 0; q < reps; q++) z |= 0.75 * x + (-1.25) * y;
  w.s("lincomb_s", (now_s() - t0) / reps);
  if (b.count("cg")) {
    TRnRelease3dSpace& x0 = vec_from(s, D(b, "x0"));
    TRnRelease3dSpace& rhs = vec_from(s, D(b, "b"));
    TSLAE* slae = new TSLAE(A, x0, rhs);
    t0 = now_s();
    slae->SolveByConjugateGradients();
    w.s("cg_s", now_s() - t0);
    TRnRelease3dSpace& res = dynamic_cast<TRnRelease3dSpace&>(const_cast<TRnSpace&>((const TRnSpace&)slae->Result));
    TRnRelease3dSpace& r = *(new TRnRelease3dSpace(s.model));
    r |= ((TRnLinearOperator&)A)(res) - rhs;
    w.s("cg_resid_l2", r.Norma(0));
  }
}

int main(int argc, char** argv) {
  if (argc != 4) { fprintf(stderr, "usage: ref_driver task in out\n"); return 2; }
  try {
    Bag b = read_bag(argv[2]);
    Writer w(argv[3]);
    std::string t = argv[1];
    if (t == "matvec") task_matvec(b, w);
    else if (t == "solve") task_solve(b, w);
    else if (t == "thomas") task_thomas(b, w);
    else if (t == "ib") task_ib(b, w);
    else if (t == "pack") task_pack(b, w);
    else if (t == "npy") task_npy(b, argv[3]);
    else if (t == "step") task_step(b, w);
    else if (t == "timing") task_timing(b, w);
    else { fprintf(stderr, "unknown task\n"); return 2; }
  } catch (const char* e) {
    fprintf(stderr, "reference threw: %s\n", e); return 3;
  } catch (std::exception& e) {
    fprintf(stderr, "driver error: %s\n", e.what()); return 4;
  }
  return 0;
}
