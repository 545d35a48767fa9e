// The drop-in for the reference's TSLAE (XSLAE.h:12-35, XSLAE.cpp): the same
// class, built from the reference's unchanged header, with every solve run on
// the GPU through include/xflow.h.  A maintainer links this file in place of
// XSLAE.cpp (and libxflow.so); the time loop's call sites stay as they are
// (XProblem.cpp:5570-5588: TSLAE(*APtr, p, rightPart), UpdateRP, UpdateP,
// SolveByBiConjugateGradientsStab, p |= Result).
//
//   g++ -std=c++11 -I<reference tree> -Iinclude -Ixflow_gb300/host -c xslae_gpu.cpp
//
// What is kept from the reference: the constructors' and destructor's
// ownership (the system deletes A, x, b and the result, XSLAE.cpp:21-30), the
// warm start from x (UpdateP), the result left in Result on the active cells
// and x unchanged, the algorithms and stopping rules of CG, BiCG, MinRes and
// BiCGStab (the C ABI's XF_CG_REFERENCE, XF_BICG, XF_MINRES, XF_BICGSTAB), and
// `throw "..."` for every failure.  The operator must be a
// T3dLaplaceOperator or T3dVariableDivergentedOperator on a T3dNormalGrid
// and the vectors its box spaces (TRnRelease3dSpace): the pressure systems of
// the time loop.  Other operators throw; the reference's CPU path is not a
// fallback.  TSLAE::SolveByScalarRunning runs one line on the GPU per call
// (the batched xf_thomas_lines is the fast form); the dense Gauss solves are
// not on the path and throw.
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "XGrid.h"
#include "XOperator.h"
#include "XSLAE.h"
#include "XSpace.h"
#include "xf_box_system.h"

namespace {

// T3dLaplaceOperator::fGrid is protected: a pointer to it formed through a
// derived class reads it on any operator.
struct LaplacePeek : T3dLaplaceOperator {
  static const T3dNormalGrid* T3dLaplaceOperator::*grid() { return &LaplacePeek::fGrid; }
};
// T3dVariableDivergentedOperator::density is private (XOperator.h:422): an
// explicit instantiation may name it (access checks do not apply there).
template <typename Tag, typename Tag::type M>
struct Expose {
  friend typename Tag::type member_of(Tag) { return M; }
};
struct DensityTag {
  typedef double*** T3dVariableDivergentedOperator::*type;
  friend type member_of(DensityTag);
};
template struct Expose<DensityTag, &T3dVariableDivergentedOperator::density>;
struct SlaePeek : TSLAE {
  static const TRnLinearOperator* TSLAE::*a() { return &SlaePeek::fA; }
};

xflow::BoxSystem& system() {
  static xflow::BoxSystem sys(0);   // one CUDA context for the process
  return sys;
}

// The system of A on its grid, x and b as boxes; the solution into result.
void solve_on_gpu(const TRnLinearOperator* A, TRnSpace* x, TRnSpace* b, TRnSpace* result, int method) {
  const T3dLaplaceOperator* lap = dynamic_cast<const T3dLaplaceOperator*>(A);
  if (!lap) throw "Error in TSLAE (xflow): the GPU solves T3dLaplaceOperator and T3dVariableDivergentedOperator systems";
  const T3dVariableDivergentedOperator* vd = dynamic_cast<const T3dVariableDivergentedOperator*>(A);
  const T3dNormalGrid& g = *(lap->*LaplacePeek::grid());
  const int n1 = g.GetSeparator1().EndIndex + 1, n2 = g.GetSeparator2().EndIndex + 1,
            n3 = g.GetSeparator3().EndIndex + 1;
  const size_t n = (size_t)n1 * n2 * n3;
  std::vector<int32_t> codes(n);
  std::vector<double> normals(3 * n, 0.0), xb(n), bb(n);
  const T3dNumberMask& mask = g.Mask;
  const T3dVector* const* const* const* nrm = g.Normals;
  TRnRelease3dSpace* xs = dynamic_cast<TRnRelease3dSpace*>(x);
  TRnRelease3dSpace* bs = dynamic_cast<TRnRelease3dSpace*>(b);
  TRnRelease3dSpace* rs = dynamic_cast<TRnRelease3dSpace*>(result);
  if (!xs || !bs || !rs) throw "Error in TSLAE (xflow): the vectors must be TRnRelease3dSpace boxes";
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) {
        const size_t c = ((size_t)i * n2 + j) * n3 + k;
        codes[c] = mask[i][j][k];
        if (const T3dVector* v = nrm[i][j][k]) {
          normals[3 * c] = v->X; normals[3 * c + 1] = v->Y; normals[3 * c + 2] = v->Z;
        }
        xb[c] = (*xs)[i][j][k];
        bb[c] = (*bs)[i][j][k];
      }
  xflow::BoxSystem& sys = system();
  sys.set_grid(n1, n2, n3, codes.data(), g.GetSeparator1().Separation, g.GetSeparator2().Separation,
               g.GetSeparator3().Separation, normals.data(), vd ? XF_OP_VARDIV : XF_OP_LAPLACE);
  if (vd) {
    double*** rho = vd->*member_of(DensityTag());
    if (!rho) throw "Error in TSLAE (xflow): withDensity has not been called on the variable-density operator";
    std::vector<double> rb(n);
    for (int i = 0; i < n1; i++)
      for (int j = 0; j < n2; j++)
        for (int k = 0; k < n3; k++) rb[((size_t)i * n2 + j) * n3 + k] = rho[i][j][k];
    sys.set_density(rb.data());
  }
  sys.solve(method, xb.data(), bb.data());
  // result |= x_k (on the active cells, XSLAE.cpp:192, 334, 365, 409)
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) {
        const int m = mask[i][j][k];
        const bool active = m == 1 || m == 4 || m == 5 || m == 6 || m == 8;   // XProblem.cpp:4155-4182
        if (active) (*rs)[i][j][k] = xb[((size_t)i * n2 + j) * n3 + k];
      }
}

}  // namespace

TSLAE::TSLAE(const TRnLinearOperator& lA, TRnSpace& lx, TRnSpace& lb) : fA(&lA), fx(&lx), fb(&lb), Result(this) {
  fResult = &lx.Copy();
  *fResult |= 0;
}
TSLAE::TSLAE(const TRnLinearOperator& lA, TRnSpace& lx, TRnSpace& lu, TRnSpace& lv, TRnSpace& lw, TRnSpace& lb)
    : fA(&lA), fx(&lx), fu(&lu), fv(&lv), fw(&lw), fb(&lb), Result(this) {
  fResult = &lx.Copy();
  *fResult |= 0;
}
TSLAE::~TSLAE() {   // the reference's ownership: the system owns its operator, vectors and result
  if (fA != NULL) delete fA;
  if (fx != NULL) delete fx;
  if (fu != NULL) delete fu;
  if (fv != NULL) delete fv;
  if (fw != NULL) delete fw;
  if (fb != NULL) delete fb;
  if (fResult != NULL) delete fResult;
}
const TRnSpace& TSLAE::GetResult() const { return *fResult; }
void TSLAE::UpdateP(TRnSpace& lp) { fx->Assign(lp); }
void TSLAE::UpdateRP(TRnSpace& lrp) { fb->Assign(lrp); }
void TSLAE::UpdateA(TRnLinearOperator&) { throw "TSLAE::UpdateA is not implemented (as in the reference)"; }

void TSLAE::SolveByConjugateGradients() { solve_on_gpu(fA, fx, fb, fResult, XF_CG_REFERENCE); }
void TSLAE::SolveByBiConjugateGradients() { solve_on_gpu(fA, fx, fb, fResult, XF_BICG); }
void TSLAE::SolveByMinimalResiduals() { solve_on_gpu(fA, fx, fb, fResult, XF_MINRES); }
void TSLAE::SolveByBiConjugateGradientsStab() { solve_on_gpu(fA, fx, fb, fResult, XF_BICGSTAB); }

void TSLAE::SolveByGauss() { throw "TSLAE::SolveByGauss: dense solves are not on the GPU path"; }
void TSLAE::SolveByGauss(const double* const* const, const double* const, double* const, const int) {
  throw "TSLAE::SolveByGauss: dense solves are not on the GPU path";
}

// One tridiagonal line (XSLAE.cpp:416-445) on the GPU: lM + 1 unknowns.
void TSLAE::SolveByScalarRunning(int lM, double* lU, const double* lA, const double* lB, const double* lC,
                                 const double* lF) {
  xf_ctx* ctx = system().context();
  cudaStream_t st = (cudaStream_t)xf_stream(ctx);
  const size_t bytes = (size_t)(lM + 1) * 8;
  static double* dev = NULL;   // five device arrays, grown when a longer line comes
  static size_t cap = 0;
  if (cap < bytes) {
    if (dev) cudaFree(dev);
    dev = NULL;
    cap = 0;
    if (cudaMalloc((void**)&dev, 5 * bytes) != cudaSuccess) throw "TSLAE::SolveByScalarRunning: device memory";
    cap = bytes;
  }
  const size_t s = cap / 8;
  const double* host[5] = {lU, lA, lB, lC, lF};
  for (int q = 0; q < 5; q++)
    if (cudaMemcpyAsync(dev + q * s, host[q], bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
      throw "TSLAE::SolveByScalarRunning: copy";
  if (xf_thomas_lines(ctx, lM, 1, 1, 0, 0, 1, dev, dev + s, dev + 2 * s, dev + 3 * s, dev + 4 * s) != XF_OK)
    throw xf_last_error(ctx);
  if (cudaMemcpyAsync(lU, dev, bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
    throw "TSLAE::SolveByScalarRunning: copy";
}
