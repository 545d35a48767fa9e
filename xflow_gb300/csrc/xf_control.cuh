// Device-side solver control: scalar recurrences of the Krylov methods run by
// the last block of the reduction that produces their inputs, so that a
// whole solver iteration needs no host round-trip.  The scalar layout lives
// in DevScratch::scalars / iscalars.
#pragma once
#include <math.h>

#include "xf_common.cuh"

// reduction slots (each matvec uses slot and slot+1)
enum { SL_A = 0, SL_B = 2, SL_C = 4, SL_D = 6 };

// FP64 scalars
enum {
  D_RR = 32, D_RR_PREV, D_ALPHA, D_BETA, D_BB, D_THR, D_RTOL2, D_EPS,
  D_TAUK = 40, D_TAUK1, D_ALFAK, D_ALFAK1, D_RK1RK1, D_RKRK, D_EPSCUR, D_C1, D_C2, D_C3,
  D_PN = 52, D_PN1, D_AN, D_BN, D_WN, D_NORM,
  D_ALFA = 60, D_RR64, D_BCG_A1, D_RZ
};
// integer scalars
// I_PAUSE: the mixed CG's inner recursion has met the tolerance (or the cap)
// and waits for the true-residual replacement at the end of its chunk.
// I_PBUF: which of the two direction buffers holds the current p (fused FP32
// iteration).  I_ERR: a bounded wait in a staged kernel ran out.  I_PFIRST:
// the preconditioned CG's next (r, z) starts the direction (beta = 0).
enum { I_DONE = 0, I_STATUS, I_IT, I_REPL, I_NEEDREP, I_MAXIT, I_REPEVERY, I_MIXED, I_PAUSE, I_PBUF, I_ERR, I_PFIRST };

enum {
  CTL_NONE = 0,
  CTL_CG_INIT, CTL_CG_ALPHA, CTL_CG_BETA, CTL_MIXED_REPL, CTL_CG_BETA_FLIP, CTL_CG_ALPHA_FLIP,
  CTL_RCG_INIT, CTL_RCG_TAU0, CTL_RCG_RES0, CTL_RCG_TAU, CTL_RCG_RES,
  CTL_BCGS_NORM0, CTL_BCGS_PN1, CTL_BCGS_AN, CTL_BCGS_WN, CTL_BCGS_END,
  CTL_MR_INIT, CTL_MR_ALFA, CTL_MR_RES,
  CTL_BICG_INIT, CTL_BICG_ALPHA, CTL_BICG_BETA,
  CTL_PCG_BETA, CTL_PCG_ALPHA_FLIP, CTL_PCG_RR, CTL_PCG_REPL, CTL_PCG_RR_BETA
};

template <typename T>
struct MvReq {
  const T* x = nullptr;
  T* y = nullptr;
  float* y32 = nullptr;
  const T* s = nullptr;
  const T* w = nullptr;
  int sign = 0, neg = 0, zero_inactive = 0, dot_self = 0;
  bool exact = false;
  int slot = SL_A;
  int ctl = CTL_NONE;
  int gate = 0;   // 1: run only while a true-residual replacement is pending
  int transpose = 0;   // packed operators: apply the other side (A^T when op applies A)
  int guard = 0;       // packed operators: skip once the solve is done (implied by ctl)
};

__device__ inline void finish(DevScratch* S, long long status) {
  S->iscalars[I_DONE] = 1;
  S->iscalars[I_STATUS] = status;
}

// Reliable updates of the preconditioned mixed CG: the FP32 recursion pauses
// (and the true FP64 residual replaces it at the end of the graph chunk) once
// its (r, r) has dropped by this factor since the last replacement, a 10^3
// drop of the norm.  A strong preconditioner reaches FP32's floor within one
// chunk, and continuing the direction from beyond that floor stalls.
constexpr double PCG_REPL_DROP2 = 1e-6;

// Runs in one thread (thread 0 of the last block of a reduction).
__device__ inline void control_step(DevScratch* S, int ctl) {
  double* d = S->scalars;
  long long* I = S->iscalars;
  switch (ctl) {
    case CTL_NONE: break;
    // ---- Hestenes-Stiefel CG (FP64 or mixed) --------------------------------
    case CTL_CG_INIT: {  // SL_A+1: r.r (FP64 true residual), SL_B: b.b
      double rr = d[SL_A + 1], bb = d[SL_B];
      d[D_RR] = rr; d[D_RR_PREV] = rr; d[D_BB] = bb; d[D_THR] = d[D_RTOL2] * bb;
      d[D_RR64] = rr;
      d[D_BETA] = 0.0;   // the fused iteration forms p = r + beta p from p = 0
      I[I_IT] = 0; I[I_REPL] = 0; I[I_NEEDREP] = 0; I[I_DONE] = 0; I[I_STATUS] = XF_OK; I[I_PBUF] = 0;
      I[I_PFIRST] = 1;
      if (isnan(rr)) finish(S, XF_NAN);
      else if (rr <= d[D_THR]) finish(S, XF_OK);
      break;
    }
    case CTL_CG_ALPHA_FLIP:  // fused direction update: the new p lives in the other buffer
      I[I_PBUF] ^= 1;
      // fall through
    case CTL_CG_ALPHA: {  // SL_A: p.q
      double pq = d[SL_A];
      if (isnan(pq)) finish(S, XF_NAN);
      else if (!(pq > 0.0)) finish(S, XF_BREAKDOWN);
      else d[D_ALPHA] = d[D_RR] / pq;
      break;
    }
    case CTL_CG_BETA_FLIP:  // fused iteration: the new p now lives in the other buffer
      I[I_PBUF] ^= 1;
      // fall through
    case CTL_CG_BETA: {  // SL_B: r.r after the update
      double rn = d[SL_B];
      I[I_IT] += 1;
      if (isnan(rn)) { finish(S, XF_NAN); break; }
      d[D_RR_PREV] = d[D_RR];
      d[D_BETA] = rn / d[D_RR];
      d[D_RR] = rn;
      if (I[I_MIXED]) {
        // the replacement at the end of the chunk confirms or resumes
        if (rn <= d[D_THR] || I[I_IT] >= I[I_MAXIT]) I[I_PAUSE] = 1;
      } else {
        if (rn <= d[D_THR]) finish(S, XF_OK);
        else if (I[I_IT] >= I[I_MAXIT]) finish(S, XF_MAXIT);
      }
      break;
    }
    case CTL_MIXED_REPL: {  // SL_C+1: true r.r in FP64
      double r64 = d[SL_C + 1];
      I[I_REPL] += 1;
      I[I_NEEDREP] = 0;
      I[I_PAUSE] = 0;
      d[D_RR64] = r64;
      if (isnan(r64)) finish(S, XF_NAN);
      else if (r64 <= d[D_THR]) finish(S, XF_OK);
      else if (I[I_IT] >= I[I_MAXIT]) finish(S, XF_MAXIT);
      else {
        d[D_BETA] = r64 / d[D_RR_PREV];
        d[D_RR] = r64;
      }
      break;
    }
    // ---- polynomially preconditioned mixed CG: rho = (r, z) ------------------
    case CTL_PCG_RR_BETA: {  // fused update + preconditioner: SL_B (r, r) after the update, SL_D (r, z)
      double rn = d[SL_B];
      I[I_IT] += 1;
      if (isnan(rn)) { finish(S, XF_NAN); break; }
      d[D_RR] = rn;
      // a paused recursion keeps the previous (r, z): the replacement's own
      // (r, z) continues the direction from it
      if (rn <= d[D_THR] || rn <= PCG_REPL_DROP2 * d[D_RR64] || I[I_IT] >= I[I_MAXIT]) { I[I_PAUSE] = 1; break; }
    }
      // fall through
    case CTL_PCG_BETA: {  // SL_D: (r, z) of the new residual
      double rz = d[SL_D];
      if (isnan(rz)) { finish(S, XF_NAN); break; }
      if (!(rz > 0.0)) { finish(S, XF_BREAKDOWN); break; }
      d[D_BETA] = I[I_PFIRST] ? 0.0 : rz / d[D_RZ];
      I[I_PFIRST] = 0;
      d[D_RZ] = rz;
      break;
    }
    case CTL_PCG_ALPHA_FLIP: {  // SL_A: (p, q); the new p lives in the other buffer
      I[I_PBUF] ^= 1;
      double pq = d[SL_A];
      if (isnan(pq)) finish(S, XF_NAN);
      else if (!(pq > 0.0)) finish(S, XF_BREAKDOWN);
      else d[D_ALPHA] = d[D_RZ] / pq;
      break;
    }
    case CTL_PCG_RR: {  // SL_B: (r, r) after the update: the inner recursion's stop test
      double rn = d[SL_B];
      I[I_IT] += 1;
      if (isnan(rn)) { finish(S, XF_NAN); break; }
      d[D_RR] = rn;
      if (rn <= d[D_THR] || rn <= PCG_REPL_DROP2 * d[D_RR64] || I[I_IT] >= I[I_MAXIT]) I[I_PAUSE] = 1;
      break;
    }
    case CTL_PCG_REPL: {  // SL_C+1: true r.r in FP64; the next (r, z) continues the direction
      double r64 = d[SL_C + 1];
      I[I_REPL] += 1;
      I[I_NEEDREP] = 0;
      I[I_PAUSE] = 0;
      d[D_RR64] = r64;
      if (isnan(r64)) finish(S, XF_NAN);
      else if (r64 <= d[D_THR]) finish(S, XF_OK);
      else if (I[I_IT] >= I[I_MAXIT]) finish(S, XF_MAXIT);
      break;
    }
    // ---- TSLAE::SolveByConjugateGradients (XSLAE.cpp:56-157) ---------------
    case CTL_RCG_INIT: {  // SL_A+1: (rk_1, rk_1)
      double v = d[SL_A + 1];
      d[D_RK1RK1] = v;
      I[I_IT] = 0; I[I_DONE] = 0; I[I_STATUS] = XF_OK;
      d[D_EPSCUR] = sqrt(v);
      if (isnan(v)) finish(S, XF_NAN);
      else if (v == 0) finish(S, XF_OK);
      break;
    }
    case CTL_RCG_TAU0: {  // SL_A: (A rk_1, rk_1)
      d[D_TAUK] = d[D_RK1RK1] / d[SL_A];
      d[D_C3] = -d[D_TAUK];
      break;
    }
    case CTL_RCG_RES0: {  // SL_A+1: (rk, rk)
      double v = d[SL_A + 1];
      d[D_RKRK] = v;
      d[D_ALFAK] = 1;
      d[D_EPSCUR] = sqrt(v);
      if (isnan(v)) finish(S, XF_NAN);
      else if (v == 0 || d[D_EPSCUR] <= d[D_EPS]) finish(S, XF_OK);
      break;
    }
    case CTL_RCG_TAU: {  // SL_A: (A rk, rk)
      double rkXrk = d[D_RKRK];
      double tauk1 = rkXrk / d[SL_A];
      double alfak1 = 1 - (1 / d[D_ALFAK]) * (tauk1 / d[D_TAUK]) * (rkXrk / d[D_RK1RK1]);
      alfak1 = 1 / alfak1;
      d[D_C1] = alfak1;
      d[D_C2] = (1 - alfak1);
      d[D_C3] = (tauk1 * alfak1);
      d[D_RK1RK1] = rkXrk;
      d[D_TAUK] = tauk1;
      d[D_ALFAK] = alfak1;
      break;
    }
    case CTL_RCG_RES: {  // SL_A+1: (rk, rk)
      double v = d[SL_A + 1];
      d[D_RKRK] = v;
      d[D_EPSCUR] = sqrt(v);
      I[I_IT] += 1;
      if (isnan(v)) finish(S, XF_NAN);
      else if (d[D_EPSCUR] <= d[D_EPS]) finish(S, XF_OK);
      else if (I[I_IT] >= I[I_MAXIT]) finish(S, XF_MAXIT);
      break;
    }
    // ---- TSLAE::SolveByBiConjugateGradientsStab (XSLAE.cpp:667-768) --------
    case CTL_BCGS_NORM0: {  // SL_D: absmax(Rn)
      d[D_PN] = 1; d[D_AN] = 1; d[D_BN] = 1; d[D_WN] = 1;
      d[D_NORM] = d[SL_D];
      I[I_IT] = 0; I[I_DONE] = 0; I[I_STATUS] = XF_OK;
      if (!(d[D_NORM] > d[D_EPS])) finish(S, isnan(d[D_NORM]) ? XF_NAN : XF_OK);
      break;
    }
    case CTL_BCGS_PN1: {  // SL_A: (sRn, Rn)
      double pn1 = d[SL_A];
      I[I_IT] += 1;
      d[D_PN1] = pn1;
      d[D_BN] = (pn1 / d[D_PN]) * (d[D_AN] / d[D_WN]);
      break;
    }
    case CTL_BCGS_AN: {  // SL_A: (sRn, Vn)
      d[D_AN] = d[D_PN1] / d[SL_A];
      break;
    }
    case CTL_BCGS_WN: {  // SL_A: (Tn, Sn), SL_A+1: (Tn, Tn)
      d[D_WN] = d[SL_A] / d[SL_A + 1];
      break;
    }
    case CTL_BCGS_END: {  // SL_D: absmax(Rn)
      d[D_PN] = d[D_PN1];
      d[D_NORM] = d[SL_D];
      if (isnan(d[D_NORM])) finish(S, XF_NAN);
      else if (!(d[D_NORM] > d[D_EPS])) finish(S, XF_OK);
      else if (I[I_IT] >= I[I_MAXIT]) finish(S, XF_MAXIT);
      break;
    }
    // ---- TSLAE::SolveByMinimalResiduals (XSLAE.cpp:350-414) ----------------
    case CTL_MR_INIT: {  // SL_A+1: (rk, rk)
      double v = d[SL_A + 1];
      d[D_RKRK] = v;
      d[D_EPSCUR] = sqrt(v);
      I[I_IT] = 0; I[I_DONE] = 0; I[I_STATUS] = XF_OK;
      if (isnan(v)) finish(S, XF_NAN);
      else if (v == 0 || d[D_EPSCUR] <= d[D_EPS]) finish(S, XF_OK);
      break;
    }
    case CTL_MR_ALFA: {  // SL_A: (Ark, rk), SL_A+1: (Ark, Ark)
      d[D_ALFA] = (-1) * d[SL_A] / d[SL_A + 1];
      I[I_IT] += 1;
      break;
    }
    case CTL_MR_RES: {  // SL_A+1: (rk, rk)
      double v = d[SL_A + 1];
      d[D_RKRK] = v;
      d[D_EPSCUR] = sqrt(v);
      if (isnan(v)) finish(S, XF_NAN);
      else if (d[D_EPSCUR] <= d[D_EPS]) finish(S, XF_OK);
      else if (I[I_IT] >= I[I_MAXIT]) finish(S, XF_MAXIT);
      break;
    }
    // ---- TSLAE::SolveByBiConjugateGradients (XSLAE.cpp:159-348) -----------
    case CTL_BICG_INIT: {  // SL_D: (rk, rk)
      double v = d[SL_D];
      d[D_EPSCUR] = sqrt(v);
      I[I_IT] = 0; I[I_DONE] = 0; I[I_STATUS] = XF_OK;
      if (isnan(v)) finish(S, XF_NAN);
      else if (!(d[D_EPSCUR] > d[D_EPS])) finish(S, XF_OK);
      break;
    }
    case CTL_BICG_ALPHA: {  // SL_B: alpha1 = (rk, rt); SL_A: alpha2 = (A pk, pt)
      I[I_IT] += 1;
      d[D_BCG_A1] = d[SL_B];
      d[D_ALPHA] = d[SL_B] / d[SL_A];
      break;
    }
    case CTL_BICG_BETA: {  // SL_C: beta1 = (rk', rt'); SL_C+1: (rk', rk')
      double beta1 = d[SL_C], beta2 = d[D_BCG_A1], rr = d[SL_C + 1];
      if (beta1 == 0 || beta2 == 0) { finish(S, XF_BREAKDOWN); break; }   // the reference throws (:274-275)
      d[D_BETA] = beta1 / beta2;
      d[D_EPSCUR] = sqrt(rr);
      if (isnan(rr) || isnan(d[D_BETA])) finish(S, XF_NAN);
      else if (!(d[D_EPSCUR] > d[D_EPS])) finish(S, XF_OK);
      else if (I[I_IT] >= I[I_MAXIT]) finish(S, XF_MAXIT);
      break;
    }
    default: break;
  }
}

// The learned two-level preconditioner's step along the prolongated coarse
// correction y: omega = (y, r) / (y, A y), 0 when (y, A y) is not positive or
// either dot is not finite.
__device__ __forceinline__ double tl_omega(const double* scal, int s_yay, int s_yr) {
  const double yay = scal[s_yay], yr = scal[s_yr];
  return (yay > 0 && isfinite(yay) && isfinite(yr)) ? yr / yay : 0.0;
}
