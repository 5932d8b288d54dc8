// Register-resident one-contact solver for the coloured NSGS sweep.
//
// Restates the reference's default local solver, OC_NSN_GP_HYBRID with
// NSN_AND_PLI_NSN_LOOP (fc3d_onecontact_nonsmooth_Newton_solvers.c:920-1015):
// a damped Alart-Curnier Newton with Goldstein-Price line search
// (:562-854), keep-or-discard on the local natural-map error (:856-918),
// then one loop of the PLI projection solver (fc3d_projection.c:350-514)
// followed by Newton again.  Everything lives in registers of the lanes that
// own the contact.
//
// The arithmetic follows the reference's operation order.  The FP64
// instantiation is compiled with --fmad=false, so it reproduces the CPU
// restatement bit for bit; the FP32 instantiation keeps FMA contraction and
// uses FP32 epsilons and tolerances (it is an accelerator, its result is
// polished in FP64).
#pragma once
#include <cfloat>
#include <cuda_runtime.h>

namespace fc3dgpu {

template <typename Real>
struct Eps;
template <>
struct Eps<double> {
  static __device__ __forceinline__ double v() { return DBL_EPSILON; }
};
template <>
struct Eps<float> {
  static __device__ __forceinline__ float v() { return FLT_EPSILON; }
};

// Square root and division of the one-contact solver (Newton, line search,
// 3x3 elimination, PLI).  They are the plain operations, except in the
// kernels built with FC3D_FAST_F64 (the opt-in fast FP64 polish), where the
// FP64 ones are refined from FP32 seeds (see below).  The natural-map error
// (projection on the cone) and rho always use the plain operations: they
// decide convergence and are stored with the layout.
template <typename Real>
__device__ __forceinline__ Real esqrt(Real x) {
  return sqrt(x);
}
template <typename Real>
__device__ __forceinline__ Real dsqrt(Real x) {
  return sqrt(x);
}
template <typename Real>
__device__ __forceinline__ Real ldiv(Real a, Real b) {
  return a / b;
}
#ifdef FC3D_FAST_F64
// One Newton-Raphson step for the reciprocal, y1 = y0 (2 - b y0) written as
// y1 = y0 + y0 (1 - b y0), from the correctly rounded FP32 reciprocal of b
// rounded to FP32: the seed's relative error e0 is below 1.2e-7, the step's
// about e0^2 < 1.5e-14, so a / b comes out within about 1.5e-14 relative
// (the exact division takes about twice as many dependent FP64 operations).
// Arguments outside the FP32 range (and zero, infinities, NaN) take the
// exact division.
template <>
__device__ __forceinline__ double ldiv<double>(double a, double b) {
  const float bf = __double2float_rn(b);
  if (!(fabsf(bf) > 1e-30f && fabsf(bf) < 1e30f)) return a / b;
  double y = (double)__frcp_rn(bf);
  const double e = fma(-b, y, 1.0);
  y = fma(y, e, y);
  return a * y;
}
// sqrt(x) from an FP32 reciprocal square root y0 by one Newton-Raphson step
// on h = x y0 (the coupled iteration sqrt(x) ~ h (1 + r / 2) with
// r = 1 - h y0): relative error about (3 e0 / 2)^2, below 1e-13 for the
// FP32 seed.  Non-positive, tiny and huge arguments take the exact root.
template <>
__device__ __forceinline__ double dsqrt<double>(double x) {
  const float xf = __double2float_rn(x);
  if (!(xf > 1e-30f && xf < 1e30f)) return sqrt(x);
  const double y = (double)rsqrtf(xf);
  const double h = x * y;
  const double r = fma(-h, y, 1.0);
  return fma(h, 0.5 * r, h);
}
#endif

// r += a v (column-major a), column by column (op3x3.h:342)
template <typename Real>
__device__ __forceinline__ void mvp3x3(const Real a[9], const Real v[3], Real r[3]) {
  r[0] += a[0] * v[0];
  r[1] += a[1] * v[0];
  r[2] += a[2] * v[0];
  r[0] += a[3] * v[1];
  r[1] += a[4] * v[1];
  r[2] += a[5] * v[1];
  r[0] += a[6] * v[2];
  r[1] += a[7] * v[2];
  r[2] += a[8] * v[2];
}

// Gaussian elimination with partial pivoting on a 3x3 column-major system
// (op3x3.h:868-980); returns nonzero when a pivot is below epsilon.
template <typename Real>
__device__ __forceinline__ int solve3x3(const Real a[9], Real b[3]) {
  const Real E = Eps<Real>::v();
  Real lp0, lp1, lp2, lm1, lm2, ln1, ln2, bl, bm, bn, f1, f2, s1, s2, alp0;
  Real a0 = a[0], a1 = a[1], a2 = a[2];
  Real aa0 = fabs(a0), aa1 = fabs(a1), aa2 = fabs(a2);
  int p1 = aa0 >= aa1 ? (aa0 >= aa2 ? 0 : 2) : (aa1 >= aa2 ? 1 : 2);
  if (p1 == 0) {
    f1 = ldiv(a1, a0); f2 = ldiv(a2, a0); lp0 = a0; alp0 = fabs(a0); lp1 = a[3]; lp2 = a[6];
    lm1 = a[4] - f1 * lp1; lm2 = a[7] - f1 * lp2; ln1 = a[5] - f2 * lp1; ln2 = a[8] - f2 * lp2;
    bl = b[0]; bm = b[1] - f1 * bl; bn = b[2] - f2 * bl;
  } else if (p1 == 1) {
    f1 = ldiv(a0, a1); f2 = ldiv(a2, a1); lp0 = a1; alp0 = fabs(a1); lp1 = a[4]; lp2 = a[7];
    lm1 = a[3] - f1 * lp1; lm2 = a[6] - f1 * lp2; ln1 = a[5] - f2 * lp1; ln2 = a[8] - f2 * lp2;
    bl = b[1]; bm = b[0] - f1 * bl; bn = b[2] - f2 * bl;
  } else {
    f1 = ldiv(a0, a2); f2 = ldiv(a1, a2); lp0 = a2; alp0 = fabs(a2); lp1 = a[5]; lp2 = a[8];
    lm1 = a[3] - f1 * lp1; lm2 = a[6] - f1 * lp2; ln1 = a[4] - f2 * lp1; ln2 = a[7] - f2 * lp2;
    bl = b[2]; bm = b[0] - f1 * bl; bn = b[1] - f2 * bl;
  }
  if (alp0 <= E) return 1;
  Real alm1 = fabs(lm1), aln1 = fabs(ln1);
  if (alm1 >= aln1) {
    if (alm1 < E) return 1;
    f1 = ldiv(ln1, lm1);
    s2 = ldiv(bn - f1 * bm, ln2 - f1 * lm2);
    s1 = ldiv(bm - lm2 * s2, lm1);
  } else {
    if (aln1 < E) return 1;
    f1 = ldiv(lm1, ln1);
    s2 = ldiv(bm - f1 * bn, lm2 - f1 * ln2);
    s1 = ldiv(bn - ln2 * s2, ln1);
  }
  b[0] = ldiv(bl - s1 * lp1 - s2 * lp2, lp0);
  b[1] = s1;
  b[2] = s2;
  return 0;
}

// projection on the Coulomb cone of coefficient mu (projectionOnCone.c:32-49)
template <typename Real>
__device__ __forceinline__ void project_cone(Real r[3], Real mu) {
  Real normT = esqrt(r[1] * r[1] + r[2] * r[2]);
  if (mu * normT <= -r[0]) {
    r[0] = 0;
    r[1] = 0;
    r[2] = 0;
  } else if (normT <= mu * r[0]) {
  } else {
    Real mu2 = mu * mu;
    r[0] = (mu * normT + r[0]) / (mu2 + Real(1));
    r[1] = mu * r[0] * r[1] / normT;
    r[2] = mu * r[0] * r[2] / normT;
  }
}

// squared natural-map error of one contact (fc3d_compute_error.c:42-56)
template <typename Real>
__device__ __forceinline__ Real unitary_error2(const Real r[3], const Real u[3], Real mu) {
  Real w[3];
  w[0] = r[0] - u[0] - mu * esqrt(u[1] * u[1] + u[2] * u[2]);
  w[1] = r[1] - u[1];
  w[2] = r[2] - u[2];
  project_cone(w, mu);
  w[0] = r[0] - w[0];
  w[1] = r[1] - w[1];
  w[2] = r[2] - w[2];
  return w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
}

// Alart-Curnier function, STD variant (fc3d_AlartCurnier_functions.c:506-646)
template <typename Real, bool GRAD>
__device__ __forceinline__ void ac_std(const Real R[3], const Real v[3], Real mu, Real rhoN, Real rhoT, Real F[3],
                                       Real A[9], Real B[9]) {
  Real RVN = R[0] - rhoN * v[0];
  Real RVT = R[1] - rhoT * v[1];
  Real RVS = R[2] - rhoT * v[2];
  Real RV = dsqrt(RVT * RVT + RVS * RVS);
  Real Radius;
  if (GRAD) {
    A[3] = 0; A[6] = 0; A[1] = 0; A[2] = 0;
    B[3] = 0; B[6] = 0; B[1] = 0; B[2] = 0;
  }
  if (RVN > Real(0)) {
    Radius = mu * RVN;
    F[0] = rhoN * v[0];
    if (GRAD) { A[0] = rhoN; B[0] = 0; }
  } else {
    Radius = 0;
    F[0] = R[0];
    if (GRAD) { A[0] = 0; B[0] = 1; }
  }
  if (RV <= Radius) {
    F[1] = rhoT * v[1];
    F[2] = rhoT * v[2];
    if (GRAD) {
      A[4] = rhoT; A[7] = 0; A[5] = 0; A[8] = rhoT;
      B[1] = 0; B[4] = 0; B[7] = 0; B[2] = 0; B[5] = 0; B[8] = 0;
    }
  } else if (RV > Radius) {
    if (Radius > Real(0)) {
      Real RV1 = ldiv(Real(1), RV);
      F[1] = R[1] - Radius * RVT * RV1;
      F[2] = R[2] - Radius * RVS * RV1;
      if (GRAD) {
        Real RV3 = RV1 * RV1 * RV1;
        Real GTT = RV1 - RVT * RVT * RV3;
        Real GTS = -RVT * RVS * RV3;
        Real GST = GTS;
        Real GSS = RV1 - RVS * RVS * RV3;
        A[1] = mu * rhoN * RVT * RV1;
        A[2] = mu * rhoN * RVS * RV1;
        A[4] = GTT * rhoT * Radius;
        A[7] = GTS * rhoT * Radius;
        A[5] = GST * rhoT * Radius;
        A[8] = GSS * rhoT * Radius;
        B[1] = -mu * RVT * RV1;
        B[4] = Real(1) - GTT * Radius;
        B[7] = -GTS * Radius;
        B[2] = -mu * RVS * RV1;
        B[5] = -GST * Radius;
        B[8] = Real(1) - GSS * Radius;
      }
    } else {
      F[1] = R[1];
      F[2] = R[2];
      if (GRAD) {
        A[4] = 0; A[7] = 0; A[5] = 0; A[8] = 0;
        B[1] = 0; B[4] = 1; B[7] = 0; B[2] = 0; B[5] = 0; B[8] = 1;
      }
    }
  }
}

template <typename Real>
struct LocalProblem {
  Real M[9];
  Real q[3];
  Real mu, rhoN, rhoT;
  Real rho_pli;  // PLI step, persists across sweeps
  Real tol;
  int newton_max, pli_max, ls_max;
  int mode;       // 0: the reference's hybrid; 1: damped Newton only
  Real residual;  // SOLVER_RESIDUAL of the local options
  int n_newton, n_pli, n_ls;  // work counters
};

template <typename Real>
__device__ __forceinline__ Real local_error(const LocalProblem<Real>& L, const Real r[3]) {
  Real nq = dsqrt(((Real(0) + L.q[0] * L.q[0]) + L.q[1] * L.q[1]) + L.q[2] * L.q[2]);
  Real v[3] = {L.q[0], L.q[1], L.q[2]};
  mvp3x3(L.M, r, v);
  Real e = Real(0) + unitary_error2(r, v, L.mu);
  e = dsqrt(e);
  if (fabs(nq) > Eps<Real>::v()) e = ldiv(e, nq);
  return e;
}

template <typename Real>
__device__ __forceinline__ Real line_search_gp(LocalProblem<Real>& L, const Real r[3], const Real dR[3],
                                               Real F[3], const Real A[9], const Real B[9], Real v[3]) {
  Real alpha = 1, amin = 0, amax = Real(1e20);
  const Real inf = Real(1e20), m1 = Real(0.1), m2 = Real(0.9);
  const Real* M = L.M;
  Real q0 = Real(0.5) * (((Real(0) + F[0] * F[0]) + F[1] * F[1]) + F[2] * F[2]);
  Real AWB[9], tmp[3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      Real s = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) s += A[i + 3 * k] * M[k + j * 3];
      AWB[i + 3 * j] = s + B[i + 3 * j];
    }
#pragma unroll
  for (int i = 0; i < 3; i++) {
    Real s = 0;
#pragma unroll
    for (int j = 0; j < 3; j++) s += AWB[i + 3 * j] * dR[j];
    tmp[i] = s;
  }
  Real dqdt0 = 0;
#pragma unroll
  for (int i = 0; i < 3; i++) dqdt0 += F[i] * tmp[i];
  for (int it = 0; it < L.ls_max; it++) {
    L.n_ls++;
#pragma unroll
    for (int i = 0; i < 3; i++) tmp[i] = r[i] + alpha * dR[i];
#pragma unroll
    for (int i = 0; i < 3; i++) v[i] = M[i] * tmp[0] + L.q[i] + M[i + 3] * tmp[1] + M[i + 6] * tmp[2];
    ac_std<Real, false>(tmp, v, L.mu, L.rhoN, L.rhoT, F, nullptr, nullptr);
    Real qv = Real(0.5) * (((Real(0) + F[0] * F[0]) + F[1] * F[1]) + F[2] * F[2]);
    Real slope = ldiv(qv - q0, alpha);
    bool C1 = (slope >= m2 * dqdt0), C2 = (slope <= m1 * dqdt0);
    if (C1 && C2) return alpha;
    if (!C1)
      amin = alpha;
    else
      amax = alpha;
    if (alpha < inf)
      alpha = Real(0.5) * (amin + amax);
    else
      alpha = 10 * alpha;
  }
  return alpha;
}

template <typename Real>
__device__ __forceinline__ void newton_damped(LocalProblem<Real>& L, Real r[3]) {
  const Real E = Eps<Real>::v();
  Real nq = dsqrt(L.q[0] * L.q[0] + L.q[1] * L.q[1] + L.q[2] * L.q[2]);
  Real nrel = 1;
  if (nq > E) nrel = ldiv(nrel, nq);
  Real dR[3], F[3] = {0, 0, 0}, A[9], B[9], AWB[9];
#pragma unroll
  for (int e = 0; e < 9; e++) { A[e] = 0; B[e] = 0; }
  Real v[3] = {L.q[0], L.q[1], L.q[2]};
  mvp3x3(L.M, r, v);
  Real t = 1;
  ac_std<Real, false>(r, v, L.mu, L.rhoN, L.rhoT, F, nullptr, nullptr);
  L.residual = dsqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2]) * nrel;
  if (L.residual < L.tol) return;
  for (int inew = 1; inew < L.newton_max; ++inew) {
    L.n_newton++;
    ac_std<Real, true>(r, v, L.mu, L.rhoN, L.rhoT, F, A, B);
    // AWB = -(A M + B), as mm3x3 + add3x3 + scal3x3
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        AWB[i + 3 * j] = -((A[i] * L.M[3 * j] + A[i + 3] * L.M[1 + 3 * j] + A[i + 6] * L.M[2 + 3 * j]) + B[i + 3 * j]);
    dR[0] = F[0];
    dR[1] = F[1];
    dR[2] = F[2];
    int info3 = solve3x3(AWB, dR);
    if (info3) {
      dR[0] = 0;
      dR[1] = 0;
      dR[2] = 0;
    } else {
      t = line_search_gp(L, r, dR, F, A, B, v);
    }
    r[0] = r[0] + t * dR[0];
    r[1] = r[1] + t * dR[1];
    r[2] = r[2] + t * dR[2];
    v[0] = L.q[0];
    v[1] = L.q[1];
    v[2] = L.q[2];
    mvp3x3(L.M, r, v);
    ac_std<Real, false>(r, v, L.mu, L.rhoN, L.rhoT, F, nullptr, nullptr);
    L.residual = dsqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2]) * nrel;
    if (info3) break;
    if (L.residual < L.tol) return;
    if (dsqrt(dR[0] * dR[0] + dR[1] * dR[1] + dR[2] * dR[2]) < 10 * E) return;
  }
}

template <typename Real>
__device__ __forceinline__ void pli_solve(LocalProblem<Real>& L, Real r[3]) {
  const Real* M = L.M;
  const Real mu = L.mu;
  Real rho = L.rho_pli, rho_k = rho;
  Real vel[3] = {0, 0, 0}, vel_k[3], r_k[3];
  Real localerror = 1, localerror_k, a1 = 0, a2 = 0;
  const Real tau = Real(2.0) / Real(3.0), tauinv = Real(3.0) / Real(2.0), Lc = Real(0.9), Lmin = Real(0.3);
  int localiter = 0;
  while ((localerror > L.tol) && (localiter < L.pli_max)) {
    localiter++;
    L.n_pli++;
    localerror_k = localerror;
    r_k[0] = r[0];
    r_k[1] = r[1];
    r_k[2] = r[2];
#pragma unroll
    for (int i = 0; i < 3; i++) vel_k[i] = M[i] * r[0] + L.q[i] + M[i + 3] * r[1] + M[i + 6] * r[2];
    int ls = 0;
    bool success = false;
    rho_k = ldiv(rho, tau);
    Real normUT = dsqrt(vel_k[1] * vel_k[1] + vel_k[2] * vel_k[2]);
    while (!success && (ls < 10)) {
      rho_k = rho_k * tau;
      r[0] = r_k[0] - rho_k * (vel_k[0] + mu * normUT);
      r[1] = r_k[1] - rho_k * vel_k[1];
      r[2] = r_k[2] - rho_k * vel_k[2];
      project_cone(r, mu);
#pragma unroll
      for (int i = 0; i < 3; i++) vel[i] = M[i] * r[0] + L.q[i] + M[i + 3] * r[1] + M[i + 6] * r[2];
      a1 = dsqrt((vel_k[0] - vel[0]) * (vel_k[0] - vel[0]) + (vel_k[1] - vel[1]) * (vel_k[1] - vel[1]) +
                 (vel_k[2] - vel[2]) * (vel_k[2] - vel[2]));
      a2 = dsqrt((r_k[0] - r[0]) * (r_k[0] - r[0]) + (r_k[1] - r[1]) * (r_k[1] - r[1]) +
                 (r_k[2] - r[2]) * (r_k[2] - r[2]));
      success = (rho_k * a1 <= Lc * a2);
      ls++;
    }
    localerror = Real(0) + unitary_error2(r, vel, mu);
    if ((rho_k * a1 < Lmin * a2) && (localerror < localerror_k))
      rho = rho_k * tauinv;
    else
      rho = rho_k;
  }
  L.rho_pli = rho;
  L.residual = localerror;
}

template <typename Real>
__device__ __forceinline__ void keep_or_discard(LocalProblem<Real>& L, Real r[3], Real rb[3], Real& cur) {
  Real e = local_error(L, r);
  bool bad = isnan(L.residual) || isinf(L.residual);
  if (!bad && (e <= L.tol || e <= cur)) {
    cur = e;
    rb[0] = r[0];
    rb[1] = r[1];
    rb[2] = r[2];
  } else {
    r[0] = rb[0];
    r[1] = rb[1];
    r[2] = rb[2];
  }
}

// fc3d_onecontact_nonsmooth_Newton_solvers_solve (onecontact.c:221-290) with
// the hybrid strategy; r holds the contact's current reaction on entry.
template <typename Real>
__device__ __forceinline__ void local_solve(LocalProblem<Real>& L, Real r[3]) {
  if (L.q[0] > -Eps<Real>::v()) {
    r[0] = 0;
    r[1] = 0;
    r[2] = 0;
    L.residual = 0;
    return;
  }
  if (L.mode == 1) {
    // accelerator mode of the FP32 sweeps: the damped Newton alone, from
    // the contact's current reaction, with no natural-map error evaluations,
    // no keep-or-discard and no PLI loop; a non-finite result keeps the
    // incoming reaction.  The FP64 polish runs the reference's hybrid.
    const Real r0[3] = {r[0], r[1], r[2]};
    newton_damped(L, r);
    if (!(isfinite(r[0]) && isfinite(r[1]) && isfinite(r[2]))) {
      r[0] = r0[0];
      r[1] = r0[1];
      r[2] = r0[2];
    }
    return;
  }
  Real rb[3] = {r[0], r[1], r[2]};
  Real cur = local_error(L, r);
  newton_damped(L, r);
  keep_or_discard(L, r, rb, cur);
  if (cur <= L.tol) {
    L.residual = cur;
    return;
  }
  if (cur >= L.tol) {
    pli_solve(L, r);
    keep_or_discard(L, r, rb, cur);
    if (!(cur < L.tol)) {
      newton_damped(L, r);
      keep_or_discard(L, r, rb, cur);
    }
  }
  L.residual = cur;
}

// rho from the diagonal block, split spectral norm strategy
// (fc3d_AlartCurnier_functions.c:784-812)
template <typename Real>
__device__ __forceinline__ void ac_rho(const Real M[9], Real& rhoN, Real& rhoT) {
  Real sw = M[1 + 1 * 3] + M[2 + 2 * 3];
  Real dw = sw * sw - Real(4.0) * (sw - M[2 + 1 * 3] + M[1 + 2 * 3]);
  if (dw > Real(0))
    dw = esqrt(dw);
  else
    dw = 0;
  rhoN = Real(1.0) / M[0];
  rhoT = Real(2.0) / (sw + dw);
}

}  // namespace fc3dgpu
