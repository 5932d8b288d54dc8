// Coloured NSGS for 3D rolling friction on the GPU (include/rfc3dgpu.h).
//
// Layout: contacts permuted by colour (stable in contact order); per permuted
// row its blocks sorted by (original) column, the column stored permuted,
// each a 5x5 column-major block; q, mu, mu_r, rho, r, u in permuted order.
// One cooperative launch runs every sweep: a colour's contacts are spread
// over all threads of the grid, a grid barrier separates colours, and the
// convergence logic runs on the device with the same bits in every block.
// FP64 without FMA contraction, in the reference's operation order; in mixed
// precision FP32 sweeps of the same loop run first and the FP64 loop starts
// from their iterate.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "rfc3dgpu.h"

extern "C" void fc3dgpu_set_error(const char* fmt, ...);

namespace rfc3dgpu {

namespace cg = cooperative_groups;

constexpr int NT = 128;
constexpr int MAXC = 128;
constexpr int TRACE_CAP = 1 << 16;
constexpr int MAX_BLOCKS = 1024;

// Kernel arguments; Real = double for the reference's loop, float for the
// FP32 sweeps that precede it in mixed precision.
template <typename Real>
struct ArgsT {
  int nc, ncol;
  const int* cptr;  // ncol + 1 permuted-row bounds of the colours
  const int* rp;    // nc + 1 slot pointer per permuted row
  const int* col;   // permuted column of each slot (slots in ascending original column)
  const int* dpos;  // offset in the row of its first diagonal block
  const Real* W;    // 25 per slot
  const Real* q;
  const Real* mu;
  const Real* mur;
  const Real* rho;
  Real* r;
  double* u;
  double norm_q, tol, local_tol;
  int local_max, max_iter;
  double* part;   // 2 slots x MAX_BLOCKS x 4 block partial sums
  double* trace;  // per-sweep light error, from trace[0]
  double* out;    // [0] sweeps, [1] final error, [2] info, [3] last light error
  int trace_cap;  // entries of trace this launch may write
  // FP32 sweeps only: their stop rules on the light error
  double switch_tol;
  int stall_window;
};
using Args = ArgsT<double>;

#define E(M, i, j) (M)[(i) + 5 * (j)]

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

// ---- 5x5 algebra in the reference's operation order (op5x5.h) -------------

template <typename Real>
__device__ __forceinline__ void mvp5(const Real* a, const Real* v, Real* r) {
#pragma unroll
  for (int j = 0; j < 5; j++)
#pragma unroll
    for (int i = 0; i < 5; i++) r[i] += a[i + 5 * j] * v[j];
}

template <typename Real>
__device__ __forceinline__ void mm5(const Real* a, const Real* b, Real* c) {
#pragma unroll
  for (int j = 0; j < 5; j++)
#pragma unroll
    for (int i = 0; i < 5; i++)
      E(c, i, j) = E(a, i, 0) * E(b, 0, j) + E(a, i, 1) * E(b, 1, j) + E(a, i, 2) * E(b, 2, j) +
                   E(a, i, 3) * E(b, 3, j) + E(a, i, 4) * E(b, 4, j);
}

// solve_5x5_gepp_for_loop (op5x5.h:642-700): b unchanged on a tiny pivot
template <typename Real>
__device__ __forceinline__ void gepp5(const Real* a, Real* b) {
  Real A[25], x[5];
#pragma unroll
  for (int i = 0; i < 25; i++) A[i] = a[i];
#pragma unroll
  for (int i = 0; i < 5; i++) x[i] = b[i];
  // fully unrolled: the row multipliers of one pivot step are independent
  // divisions, issued together
#pragma unroll
  for (int i = 0; i < 5; i++) {
    int p = i;
    Real best = fabs(E(A, i, i));
#pragma unroll
    for (int k = i + 1; k < 5; k++)
      if (fabs(E(A, k, i)) > best) {
        best = fabs(E(A, k, i));
        p = k;
      }
    if (best < Real(1e-16)) return;
    if (p != i) {
      // swap rows i and p (p > i), with register-resident indexing
#pragma unroll
      for (int k = i + 1; k < 5; k++)
        if (k == p) {
#pragma unroll
          for (int j = 0; j < 5; j++) {
            const Real t = E(A, i, j);
            E(A, i, j) = E(A, k, j);
            E(A, k, j) = t;
          }
          const Real t = x[i];
          x[i] = x[k];
          x[k] = t;
        }
    }
    Real f[5];
#pragma unroll
    for (int k = i + 1; k < 5; k++) f[k] = E(A, k, i) / E(A, i, i);
#pragma unroll
    for (int k = i + 1; k < 5; k++) {
#pragma unroll
      for (int j = i; j < 5; j++) E(A, k, j) -= f[k] * E(A, i, j);
      x[k] -= f[k] * x[i];
    }
  }
#pragma unroll
  for (int i = 4; i >= 0; i--) {
    Real s = 0;
#pragma unroll
    for (int j = i + 1; j < 5; j++) s += E(A, i, j) * x[j];
    x[i] = (x[i] - s) / E(A, i, i);
  }
#pragma unroll
  for (int i = 0; i < 5; i++) b[i] = x[i];
}

// ---- the rolling cone (projectionOnRollingCone.c) ------------------------

enum { RC_DUAL = 0, RC_INSIDE, RC_FRICTION, RC_ROLLING, RC_FRICTION_ROLLING };

template <typename Real>
__device__ __forceinline__ int proj_rcone(Real* r, Real mu, Real mur) {
  const Real nT = sqrt(r[1] * r[1] + r[2] * r[2]);
  const Real nM = sqrt(r[3] * r[3] + r[4] * r[4]);
  if (mu * nT + mur * nM <= -r[0]) {
#pragma unroll
    for (int i = 0; i < 5; i++) r[i] = Real(0.0);
    return RC_DUAL;
  }
  if ((nT <= mu * r[0]) && (nM <= mur * r[0])) return RC_INSIDE;
  const Real mu2 = mu * mu, mur2 = mur * mur;
  Real t = (mu * nT + mur * nM + r[0]) / (mur2 + mu2 + Real(1.0));
  if ((nT > mu * t) && (nM > mur * t)) {
    r[0] = t;
    r[1] = mu * r[0] * r[1] / nT;
    r[2] = mu * r[0] * r[2] / nT;
    r[3] = mur * r[0] * r[3] / nM;
    r[4] = mur * r[0] * r[4] / nM;
    return RC_FRICTION_ROLLING;
  }
  t = (mu * nT + r[0]) / (mu2 + Real(1.0));
  if ((nT > mu * t) && (nM <= mur * t)) {
    r[0] = t;
    r[1] = mu * r[0] * r[1] / nT;
    r[2] = mu * r[0] * r[2] / nT;
    return RC_FRICTION;
  }
  t = (mur * nM + r[0]) / (mur2 + Real(1.0));
  if ((nT <= mu * t) && (nM > mur * t)) {
    r[0] = t;
    r[3] = mur * r[0] * r[3] / nM;
    r[4] = mur * r[0] * r[4] / nM;
    return RC_ROLLING;
  }
  return 20;
}

// subdifferentialProjectionOnRollingCone (projectionOnRollingCone.c),
// zero where the reference leaves the matrix unset
template <typename Real>
__device__ __forceinline__ void subdiff_rcone(Real* H, const Real* r, Real mu, Real mur) {
#pragma unroll
  for (int i = 0; i < 25; i++) H[i] = Real(0.0);
  const Real nT = sqrt(r[1] * r[1] + r[2] * r[2]);
  const Real nM = sqrt(r[3] * r[3] + r[4] * r[4]);
  if (mu * nT + mur * nM <= -r[0]) return;
  if ((nT <= mu * r[0]) && (nM <= mur * r[0])) {
#pragma unroll
    for (int i = 0; i < 5; i++) E(H, i, i) = Real(1.);
    return;
  }
  const Real mu2 = mu * mu, mur2 = mur * mur;
  const Real a1 = mu * nT + mur * nM + r[0];
  Real k = Real(1.) / (Real(1.) + mu2 + mur2);
  Real t = a1 * k;
  if ((nT > mu * t) && (nM > mur * t)) {
    E(H, 0, 0) = Real(1.) * k;
    const Real s1 = r[1] / nT, s2 = r[2] / nT;
    const Real mk = mu * k;
    E(H, 0, 1) = mk * s1;
    E(H, 0, 2) = mk * s2;
    const Real s3 = r[3] / nM, s4 = r[4] / nM;
    const Real rk = mur * k;
    E(H, 0, 3) = rk * s3;
    E(H, 0, 4) = rk * s4;
    E(H, 1, 0) = E(H, 0, 1);
    E(H, 2, 0) = E(H, 0, 2);
    E(H, 3, 0) = E(H, 0, 3);
    E(H, 4, 0) = E(H, 0, 4);
    const Real mkT = mk / nT, a2 = r[0] + mur * nM;
    E(H, 1, 1) = mkT * (-a2 * s1 * s1 + a1);
    E(H, 1, 2) = mkT * (-a2 * s1 * s2);
    E(H, 1, 3) = mk * s1 * mur * s3;
    E(H, 1, 4) = mk * s1 * mur * s4;
    E(H, 2, 1) = mkT * (-a2 * s1 * s2);
    E(H, 2, 2) = mkT * (-a2 * s2 * s2 + a1);
    E(H, 2, 3) = mk * s2 * mur * s3;
    E(H, 2, 4) = mk * s2 * mur * s4;
    const Real rkM = rk / nM, a3 = r[0] + mu * nT;
    E(H, 3, 3) = rkM * (-a3 * s3 * s3 + a1);
    E(H, 3, 4) = rkM * (-a3 * s3 * s4);
    E(H, 3, 1) = E(H, 1, 3);
    E(H, 3, 2) = E(H, 2, 3);
    E(H, 4, 3) = rkM * (-a3 * s3 * s4);
    E(H, 4, 4) = rkM * (-a3 * s4 * s4 + a1);
    E(H, 4, 1) = E(H, 1, 4);
    E(H, 4, 2) = E(H, 2, 4);
    return;
  }
  const Real b1 = r[0] + mu * nT;
  k = Real(1.) / (Real(1.) + mu2);
  t = b1 * k;
  if ((nT > mu * t) && (nM <= mur * t)) {
    E(H, 0, 0) = Real(1.) * k;
    const Real s1 = r[1] / nT, s2 = r[2] / nT;
    const Real mk = mu * k;
    E(H, 1, 0) = mk * s1;
    E(H, 2, 0) = mk * s2;
    E(H, 0, 1) = E(H, 1, 0);
    E(H, 0, 2) = E(H, 2, 0);
    const Real mkT = mk / nT;
    E(H, 1, 1) = mkT * (-r[0] * s1 * s1 + b1);
    E(H, 1, 2) = mkT * (-r[0] * s1 * s2);
    E(H, 2, 1) = mkT * (-r[0] * s1 * s2);
    E(H, 2, 2) = mkT * (-r[0] * s2 * s2 + b1);
    E(H, 3, 3) = Real(1.);
    E(H, 4, 4) = Real(1.);
    return;
  }
  const Real c1 = mur * nM + r[0];
  const Real kr = Real(1.) / (Real(1.) + mur2);
  t = c1 * kr;
  if ((nT <= mu * t) && (nM > mur * t)) {
    E(H, 0, 0) = Real(1.) * kr;
    const Real s3 = r[3] / nM, s4 = r[4] / nM;
    const Real rk = mur * kr;
    E(H, 3, 0) = rk * s3;
    E(H, 4, 0) = rk * s4;
    E(H, 0, 3) = E(H, 3, 0);
    E(H, 0, 4) = E(H, 4, 0);
    const Real rkM = rk / nM;
    E(H, 3, 3) = rkM * (-r[0] * s3 * s3 + c1);
    E(H, 3, 4) = rkM * (-r[0] * s3 * s4);
    E(H, 4, 3) = rkM * (-r[0] * s3 * s4);
    E(H, 4, 4) = rkM * (-r[0] * s4 * s4 + c1);
    E(H, 1, 1) = Real(1.);
    E(H, 2, 2) = Real(1.);
  }
}

// rolling_friction_3D_computeNaturalMap (rolling_naturalmap_functions.c:31-165)
template <typename Real>
__device__ __forceinline__ void natural_map(const Real* R, const Real* v, Real mu, Real mur, Real rho, Real* F,
                            Real* A, Real* B) {
  const Real nVT = sqrt(v[1] * v[1] + v[2] * v[2]);
  const Real nOT = sqrt(v[3] * v[3] + v[4] * v[4]);
  Real RV[5];
  RV[0] = R[0] - rho * (v[0] + mu * nVT + mur * nOT);
  RV[1] = R[1] - rho * v[1];
  RV[2] = R[2] - rho * v[2];
  RV[3] = R[3] - rho * v[3];
  RV[4] = R[4] - rho * v[4];
#pragma unroll
  for (int i = 0; i < 5; i++) F[i] = RV[i];
  const int where = proj_rcone<Real>(F, mu, mur);
#pragma unroll
  for (int i = 0; i < 5; i++) F[i] = R[i] - F[i];
  if (!A) return;
  if (where == RC_DUAL) {
#pragma unroll
    for (int i = 0; i < 25; i++) A[i] = Real(0.);
#pragma unroll
    for (int i = 0; i < 25; i++) B[i] = Real(0.);
#pragma unroll
    for (int i = 0; i < 5; i++) E(B, i, i) = Real(1.);
    return;
  }
  Real s1, s2, s3, s4;
  if (nVT <= Real(0.0)) {
    s1 = Real(1.);
    s2 = Real(0.);
  } else {
    s1 = v[1] / nVT;
    s2 = v[2] / nVT;
  }
  if (nOT <= Real(0.0)) {
    s3 = Real(1.);
    s4 = Real(0.);
  } else {
    s3 = v[3] / nOT;
    s4 = v[4] / nOT;
  }
  Real D[25];
#pragma unroll
  for (int i = 0; i < 25; i++) D[i] = Real(0.);
  E(D, 0, 0) = rho;
  E(D, 0, 1) = rho * mu * s1;
  E(D, 0, 2) = rho * mu * s2;
  E(D, 0, 3) = rho * mur * s3;
  E(D, 0, 4) = rho * mur * s4;
  E(D, 1, 1) = rho;
  E(D, 2, 2) = rho;
  E(D, 3, 3) = rho;
  E(D, 4, 4) = rho;
  if (where == RC_INSIDE) {
#pragma unroll
    for (int i = 0; i < 25; i++) A[i] = D[i];
#pragma unroll
    for (int i = 0; i < 25; i++) B[i] = Real(0.);
    return;
  }
  Real H[25];
  subdiff_rcone<Real>(H, RV, mu, mur);
  mm5<Real>(H, D, A);
#pragma unroll
  for (int i = 0; i < 25; i++) B[i] = Real(0.);
#pragma unroll
  for (int i = 0; i < 5; i++) E(B, i, i) = Real(1.);
#pragma unroll
  for (int i = 0; i < 25; i++) B[i] -= H[i];
}

// rolling_friction_3d_onecone_nonsmooth_Newton_solvers_solve_direct
// (rolling_friction_3d_onecone_nonsmooth_Newton_solvers.c:344-505)
template <typename Real>
__device__ __forceinline__ void local_nsn(const Real* M, const Real* q, Real mu, Real mur, Real rho, Real* r, Real tol,
                          int itermax) {
  const Real nq = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3] + q[4] * q[4]);
  Real rel = Real(1.0);
  if (nq > Eps<Real>::v()) rel /= nq;
  Real v[5], F[5], A[25], B[25], AWB[25], dR[5];
#pragma unroll
  for (int i = 0; i < 5; i++) v[i] = q[i];
  mvp5<Real>(M, r, v);
  natural_map<Real>(r, v, mu, mur, rho, F, nullptr, nullptr);
  Real res = sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3] + F[4] * F[4]) * rel;
  if (res < tol) return;
  for (int it = 1; it < itermax; it++) {
    natural_map<Real>(r, v, mu, mur, rho, F, A, B);
    mm5<Real>(A, M, AWB);
#pragma unroll
    for (int i = 0; i < 25; i++) AWB[i] += B[i];
#pragma unroll
    for (int i = 0; i < 25; i++) AWB[i] *= -Real(1.);
#pragma unroll
    for (int i = 0; i < 5; i++) dR[i] = F[i];
    gepp5<Real>(AWB, dR);
#pragma unroll
    for (int i = 0; i < 5; i++) r[i] += dR[i];
#pragma unroll
    for (int i = 0; i < 5; i++) v[i] = q[i];
    mvp5<Real>(M, r, v);
    natural_map<Real>(r, v, mu, mur, rho, F, nullptr, nullptr);
    const Real e2 = (F[0] * F[0] + F[1] * F[1] + F[2] * F[2] * F[2] + F[3] * F[3] + F[4] * F[4]) * rel;
    const Real old = res;
    res = sqrt(fmax(Real(0.0), e2));
    if (res < tol) return;
    if (fabs(res - old) < Eps<Real>::v()) return;
  }
}

// ---- grid-wide pieces ------------------------------------------------------

__device__ __forceinline__ void grid_sync(cg::grid_group& g) {
  if (gridDim.x == 1)
    __syncthreads();
  else
    g.sync();
}

struct Reduce {
  double warp[NT / 32][4];
  double bcast[4];
  int calls;
};

// Sum of N values over the grid in a fixed order (warp tree, warps in
// order, blocks in order): every block gets the same bits.  The partials go
// through a two-slot ring in global memory: a block writes slot k & 1 only
// after the barrier of call k - 1, which every block passes after reading
// call k - 2's slot.  The barrier also orders all reaction updates before it.
template <int N, typename A>
__device__ void grid_sum(double v[N], const A& a, Reduce& R, cg::grid_group& g) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < N; i++) {
    double x = v[i];
    for (int o = 16; o >= 1; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) R.warp[w][i] = x;
  }
  __syncthreads();
  double* slot = a.part + (size_t)(R.calls & 1) * MAX_BLOCKS * 4;
  if (threadIdx.x == 0) {
    for (int i = 0; i < N; i++) {
      double s = 0.0;
      for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += R.warp[k][i];
      __stcg(&slot[4 * blockIdx.x + i], s);
    }
  }
  grid_sync(g);
  if (threadIdx.x == 0) {
    for (int i = 0; i < N; i++) {
      double s = 0.0;
      for (int b = 0; b < (int)gridDim.x; b++) s += __ldcg(&slot[4 * b + i]);
      R.bcast[i] = s;
    }
    R.calls++;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < N; i++) v[i] = R.bcast[i];
  __syncthreads();
}

// rolling_friction_3d_compute_error (rolling_friction_3d_compute_error.c:
// 58-110): u = 1.0 q + 1.0 (row sums of W r in column order)
__device__ double full_error(const Args& a, Reduce& R, cg::grid_group& g) {
  double v[3] = {0.0, 0.0, 0.0};
  const int g0 = blockIdx.x * blockDim.x + threadIdx.x, G = gridDim.x * blockDim.x;
  for (int p = g0; p < a.nc; p += G) {
    double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int sl = a.rp[p]; sl < a.rp[p + 1]; sl++) {
      const int j = a.col[sl];
      const double* blk = a.W + 25 * (size_t)sl;
      double x[5];
      for (int k = 0; k < 5; k++) x[k] = __ldcg(&a.r[5 * (size_t)j + k]);
      for (int k = 0; k < 5; k++)
        for (int i = 0; i < 5; i++) s[i] += __ldg(&blk[i + 5 * k]) * x[k];
    }
    double uu[5], rr[5];
    for (int i = 0; i < 5; i++) {
      uu[i] = 1.0 * a.q[5 * (size_t)p + i] + 1.0 * s[i];
      __stcg(&a.u[5 * (size_t)p + i], uu[i]);
      rr[i] = __ldcg(&a.r[5 * (size_t)p + i]);
    }
    const double mu = a.mu[p], mur = a.mur[p];
    double t[5];
    t[0] = rr[0] - uu[0] - mu * sqrt(uu[1] * uu[1] + uu[2] * uu[2]) - mur * sqrt(uu[3] * uu[3] + uu[4] * uu[4]);
    for (int i = 1; i < 5; i++) t[i] = rr[i] - uu[i];
    proj_rcone(t, mu, mur);
    for (int i = 0; i < 5; i++) t[i] = rr[i] - t[i];
    v[0] += t[0] * t[0] + t[1] * t[1] + t[2] * t[2] + t[3] * t[3] + t[4] * t[4];
    for (int i = 0; i < 5; i++) v[1] += rr[i] * rr[i];
    for (int i = 0; i < 5; i++) v[2] += uu[i] * uu[i];
  }
  grid_sum<3>(v, a, R, g);
  double e = sqrt(v[0]);
  double norm = fmax(a.norm_q, sqrt(v[1]));
  norm = fmax(norm, sqrt(v[2]));
  if (fabs(norm) > DBL_EPSILON) e /= norm;
  return e;
}

// One sweep over the colours (rolling_friction_3d_nsgs.c:520-590 in colour
// order): per contact q_loc = q_p + the row sums over the other contacts'
// columns (in column order), the take-off shortcut or the one-contact
// Newton, the new reaction; v gets this thread's sum |r_old - r_new|^2 and
// sum |r_new|^2 (in the precision of the sweep, summed in FP64).
template <typename Real>
__device__ __forceinline__ void sweep_colours(const ArgsT<Real>& a, Real local_tol, double v[2],
                                              cg::grid_group& g) {
  const int g0 = blockIdx.x * blockDim.x + threadIdx.x, G = gridDim.x * blockDim.x;
  for (int c = 0; c < a.ncol; c++) {
    for (int p = a.cptr[c] + g0; p < a.cptr[c + 1]; p += G) {
      Real s[5] = {Real(0.0), Real(0.0), Real(0.0), Real(0.0), Real(0.0)};
      const int s0 = a.rp[p], s1 = a.rp[p + 1];
      for (int sl = s0; sl < s1; sl++) {
        const int j = a.col[sl];
        if (j == p) continue;
        const Real* blk = a.W + 25 * (size_t)sl;
        Real x[5];
        for (int k = 0; k < 5; k++) x[k] = __ldcg(&a.r[5 * (size_t)j + k]);
        for (int k = 0; k < 5; k++)
          for (int i = 0; i < 5; i++) s[i] += __ldg(&blk[i + 5 * k]) * x[k];
      }
      Real ql[5], rl[5], old[5];
      for (int i = 0; i < 5; i++) {
        ql[i] = a.q[5 * (size_t)p + i] + s[i];
        old[i] = __ldcg(&a.r[5 * (size_t)p + i]);
        rl[i] = old[i];
      }
      if (ql[0] > -Eps<Real>::v()) {
        for (int i = 0; i < 5; i++) rl[i] = Real(0.0);
      } else {
        Real M[25];
        const Real* d = a.W + 25 * (size_t)(s0 + a.dpos[p]);
        for (int i = 0; i < 25; i++) M[i] = __ldg(&d[i]);
        local_nsn<Real>(M, ql, a.mu[p], a.mur[p], a.rho[p], rl, local_tol, a.local_max);
      }
      const Real d0 = old[0] - rl[0], d1 = old[1] - rl[1], d2 = old[2] - rl[2], d3 = old[3] - rl[3],
                 d4 = old[4] - rl[4];
      v[0] += (double)(d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3 + d4 * d4);
      for (int i = 0; i < 5; i++) {
        v[1] += (double)(rl[i] * rl[i]);
        __stcg(&a.r[5 * (size_t)p + i], rl[i]);
      }
    }
    if (c + 1 < a.ncol) grid_sync(g);
  }
}

__global__ void __launch_bounds__(NT) k_rfc3d_nsgs(const Args a) {
  __shared__ Reduce R;
  cg::grid_group g = cg::this_grid();
  if (threadIdx.x == 0) R.calls = 0;
  __syncthreads();
  const int g0 = blockIdx.x * blockDim.x + threadIdx.x, G = gridDim.x * blockDim.x;
  const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
  double tolerance = a.tol, err = 1., local_tol = a.local_tol;
  int iter = 0, not_conv = 1;
  while (iter < a.max_iter && not_conv) {
    ++iter;
    double v[2] = {0.0, 0.0};
    sweep_colours<double>(a, local_tol, v, g);
    grid_sum<2>(v, a, R, g);
    err = sqrt(v[0]);
    const double nr = sqrt(v[1]);
    if (fabs(nr) > DBL_EPSILON) err /= nr;
    if (a.trace && lead && iter <= a.trace_cap) a.trace[iter - 1] = err;
    // determine_convergence_with_full_final (rolling_friction_3d_nsgs.c:243-285)
    not_conv = 1;
    if (err < tolerance) {
      not_conv = 0;
      const double full = full_error(a, R, g);
      if (full > a.tol) {
        if (err < DBL_EPSILON)
          local_tol = fmax(local_tol / 100., DBL_EPSILON * 1e-6);
        else
          tolerance = err / full * a.tol;
        not_conv = 1;
      }
    }
  }
  const double light = err;
  err = full_error(a, R, g);
  not_conv = !(err < a.tol);
  if (lead) {
    a.out[0] = iter;
    a.out[1] = err;
    a.out[2] = not_conv;
    a.out[3] = light;
  }
}

// The FP32 sweeps of mixed precision: the reference's loop in FP32 (FP64
// sums of the light error) without its full-error test, ending when the
// light error drops below switch_tol, makes no 1 % progress for
// stall_window sweeps, turns non-finite (out[2] = 1) or the budget ends.
// The FP64 loop then starts from their iterate.
__global__ void __launch_bounds__(NT) k_rfc3d_sweeps32(const ArgsT<float> a) {
  __shared__ Reduce R;
  cg::grid_group g = cg::this_grid();
  if (threadIdx.x == 0) R.calls = 0;
  __syncthreads();
  const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
  double err = INFINITY, best = INFINITY;
  int iter = 0, best_iter = 0;
  bool finite = true;
  while (iter < a.max_iter) {
    ++iter;
    double v[2] = {0.0, 0.0};
    sweep_colours<float>(a, (float)a.local_tol, v, g);
    grid_sum<2>(v, a, R, g);
    err = sqrt(v[0]);
    const double nr = sqrt(v[1]);
    if (fabs(nr) > DBL_EPSILON) err /= nr;
    if (a.trace && lead && iter <= a.trace_cap) a.trace[iter - 1] = err;
    if (!(err == err) || isinf(err)) {
      finite = false;
      break;
    }
    if (err < a.switch_tol) break;
    if (err < 0.99 * best) {
      best = err;
      best_iter = iter;
    } else if (a.stall_window > 0 && iter - best_iter >= a.stall_window) {
      break;
    }
  }
  if (lead) {
    a.out[0] = iter;
    a.out[2] = finite ? 0 : 1;
    a.out[3] = err;
  }
}

__global__ void k_rfc3d_to_f32(int n, const double* __restrict__ x, float* __restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = (float)x[i];
}

__global__ void k_rfc3d_to_f64(int n, const float* __restrict__ x, double* __restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = (double)x[i];
}

__global__ void __launch_bounds__(NT) k_rfc3d_error(const Args a) {
  __shared__ Reduce R;
  cg::grid_group g = cg::this_grid();
  if (threadIdx.x == 0) R.calls = 0;
  __syncthreads();
  const double e = full_error(a, R, g);
  if (blockIdx.x == 0 && threadIdx.x == 0) a.out[1] = e;
}

}  // namespace rfc3dgpu

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
using namespace rfc3dgpu;

// Largest eigenvalue of a symmetric 5x5 block (its lower triangle): the
// cyclic Jacobi iteration of the reference's eigvals_sym5x5_for_loop
// (linalg/op5x5.h:775-870) -- rotation angle from atan2, at most 50 sweeps,
// stop when the squared off-diagonal entries visited sum below 1e-24.  Run on
// the host with the C library's atan2, cos and sin, as the reference does.
static double max_eig5(const double* a) {
  double A[25];
  for (int j = 0; j < 5; j++)
    for (int i = 0; i < 5; i++) E(A, i, j) = i >= j ? E(a, i, j) : 0.0;
  for (int j = 0; j < 5; j++)
    for (int i = j + 1; i < 5; i++) E(A, j, i) = E(A, i, j);
  for (int sweep = 0; sweep < 50; sweep++) {
    double off = 0.0;
    for (int p = 0; p < 5; p++)
      for (int q = p + 1; q < 5; q++) {
        const double apq = E(A, q, p);
        if (fabs(apq) < 1e-12) continue;
        off += apq * apq;
        const double app = E(A, p, p), aqq = E(A, q, q);
        const double phi = 0.5 * atan2(2.0 * apq, aqq - app);
        const double c = cos(phi), s = sin(phi);
        for (int i = 0; i < 5; i++) {
          const double aip = E(A, i, p), aiq = E(A, i, q);
          E(A, i, p) = c * aip - s * aiq;
          E(A, i, q) = s * aip + c * aiq;
        }
        for (int j = 0; j < 5; j++) {
          const double apj = E(A, p, j), aqj = E(A, q, j);
          E(A, p, j) = c * apj - s * aqj;
          E(A, q, j) = s * apj + c * aqj;
        }
        E(A, p, p) = c * c * app - 2.0 * c * s * apq + s * s * aqq;
        E(A, q, q) = s * s * app + 2.0 * c * s * apq + c * c * aqq;
        E(A, q, p) = 0.0;
        E(A, p, q) = 0.0;
      }
    if (off < 1e-12 * 1e-12) break;
  }
  double m = E(A, 0, 0);
  for (int i = 1; i < 5; i++) m = std::max(m, E(A, i, i));
  return m;
}

struct rfc3dgpu_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  int nc = 0, ncol = 0, max_colour = 0, blocks = 1, threads = NT;
  double norm_q = 0.0;
  std::vector<int> perm, iperm, colour;
  std::vector<double> rho_host;
  int *cptr = nullptr, *rp = nullptr, *col = nullptr, *dpos = nullptr;
  double *W = nullptr, *q = nullptr, *mu = nullptr, *mur = nullptr, *rho = nullptr, *r = nullptr, *u = nullptr,
         *part = nullptr, *trace = nullptr, *out = nullptr;
  // FP32 copies for the FP32 sweeps of mixed precision
  float *W32 = nullptr, *q32 = nullptr, *mu32 = nullptr, *mur32 = nullptr, *rho32 = nullptr, *r32 = nullptr;
  int trace_len = 0;
  // 1: FP64 sweeps only (default); 0: FP32 sweeps, then the FP64 loop
  int precision = 1;
  double switch_tol = 0.0;  // FP32 sweeps end below this light error (0: max(tol, 1e-6))
  int stall = 64;
  int sweeps32 = 0, sweeps64 = 0;
};

// local tolerance of the FP32 one-contact Newton (the reference's 1e-12 is
// below FP32 resolution)
static const double LOCAL_TOL32 = 1e-6;

#define KR(x)                                                                             \
  do {                                                                                    \
    cudaError_t e_ = (x);                                                                 \
    if (e_ != cudaSuccess) {                                                              \
      fc3dgpu_set_error("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
      return NUMERICS_ERR_UNKNOWN;                                                        \
    }                                                                                     \
  } while (0)

static void free_problem(rfc3dgpu_ctx* c) {
  void* ptrs[] = {c->cptr, c->rp,  c->col, c->dpos, c->W,   c->q,    c->mu,    c->mur,   c->rho,
                  c->r,    c->u,   c->W32, c->q32,  c->mu32, c->mur32, c->rho32, c->r32};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  c->cptr = c->rp = c->col = c->dpos = nullptr;
  c->W = c->q = c->mu = c->mur = c->rho = c->r = c->u = nullptr;
  c->W32 = c->q32 = c->mu32 = c->mur32 = c->rho32 = c->r32 = nullptr;
  c->nc = 0;
}

extern "C" void rfc3dgpu_ctx_destroy(rfc3dgpu_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  free_problem(c);
  void* ptrs[] = {c->part, c->trace, c->out};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" rfc3dgpu_ctx* rfc3dgpu_ctx_create(int device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    fc3dgpu_set_error("rfc3dgpu_ctx_create: no CUDA device %d", device);
    return nullptr;
  }
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  if (!coop) {
    fc3dgpu_set_error("rfc3dgpu_ctx_create: device %d has no cooperative launch", device);
    return nullptr;
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    fc3dgpu_set_error("rfc3dgpu_ctx_create: cudaSetDevice(%d) failed", device);
    return nullptr;
  }
  rfc3dgpu_ctx* c = new rfc3dgpu_ctx();
  c->device = device;
  bool ok = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreate(&c->ev[0]) == cudaSuccess && cudaEventCreate(&c->ev[1]) == cudaSuccess &&
            cudaMalloc(&c->part, sizeof(double) * 2 * MAX_BLOCKS * 4) == cudaSuccess &&
            cudaMalloc(&c->trace, sizeof(double) * TRACE_CAP) == cudaSuccess &&
            cudaMalloc(&c->out, sizeof(double) * 8) == cudaSuccess;
  if (!ok) {
    fc3dgpu_set_error("rfc3dgpu_ctx_create: set-up failed (%s)", cudaGetErrorString(cudaGetLastError()));
    rfc3dgpu_ctx_destroy(c);
    return nullptr;
  }
  return c;
}

template <typename T>
static cudaError_t upload(T** d, const std::vector<T>& h) {
  cudaError_t e = cudaMalloc((void**)d, sizeof(T) * (h.empty() ? 1 : h.size()));
  if (e != cudaSuccess) return e;
  if (!h.empty()) e = cudaMemcpy(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
  return e;
}

extern "C" int rfc3dgpu_ctx_set_problem(rfc3dgpu_ctx* c, int nc, const int64_t* rowptr, const int64_t* colidx,
                                        const double* blocks, const double* q, const double* mu, const double* mur,
                                        int colour_kind) {
  if (!c || nc <= 0 || !rowptr || !colidx || !blocks || !q || !mu || !mur) {
    fc3dgpu_set_error("rfc3dgpu_ctx_set_problem: invalid argument");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  const int64_t nnzb = rowptr[nc];
  if (rowptr[0] != 0 || nnzb < nc || nnzb > INT32_MAX / 25) {
    fc3dgpu_set_error("rfc3dgpu_ctx_set_problem: bad row pointer");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  for (int i = 0; i < nc; i++) {
    if (rowptr[i + 1] < rowptr[i]) {
      fc3dgpu_set_error("rfc3dgpu_ctx_set_problem: row pointer decreases at %d", i);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
    bool diag = false;
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
      if (colidx[k] < 0 || colidx[k] >= nc) {
        fc3dgpu_set_error("rfc3dgpu_ctx_set_problem: column index %lld out of range", (long long)colidx[k]);
        return NUMERICS_ERR_INVALID_ARGUMENT;
      }
      diag = diag || colidx[k] == i;
    }
    if (!diag) {
      fc3dgpu_set_error("rfc3dgpu_ctx_set_problem: contact %d has no diagonal block", i);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
    if (!(mu[i] >= 0.0) || isinf(mu[i]) || !(mur[i] >= 0.0) || isinf(mur[i])) {
      fc3dgpu_set_error("rfc3dgpu_ctx_set_problem: mu[%d] = %g, mu_r[%d] = %g are not friction coefficients", i,
                        mu[i], i, mur[i]);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
  }
  std::vector<int32_t> colour(nc);
  const int ncol = fc3dgpu_colour(nc, rowptr, colidx, colour_kind ? colour_kind : FC3DGPU_COLOURING_DEFAULT,
                                  colour.data());
  if (ncol < 0) return ncol;
  if (ncol > MAXC) {
    fc3dgpu_set_error("rfc3dgpu_ctx_set_problem: %d colours (at most %d)", ncol, MAXC);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (cudaSetDevice(c->device) != cudaSuccess) {
    fc3dgpu_set_error("rfc3dgpu_ctx_set_problem: cudaSetDevice failed");
    return NUMERICS_ERR_UNKNOWN;
  }
  free_problem(c);
  c->colour.assign(colour.begin(), colour.end());
  c->perm.resize(nc);
  std::iota(c->perm.begin(), c->perm.end(), 0);
  std::stable_sort(c->perm.begin(), c->perm.end(), [&](int x, int y) { return colour[x] < colour[y]; });
  c->iperm.resize(nc);
  for (int p = 0; p < nc; p++) c->iperm[c->perm[p]] = p;
  std::vector<int> cptr(ncol + 1, 0);
  for (int i = 0; i < nc; i++) cptr[colour[i] + 1]++;
  for (int k = 0; k < ncol; k++) cptr[k + 1] += cptr[k];
  std::vector<int> rp(nc + 1, 0), col((size_t)nnzb), dpos(nc);
  std::vector<double> W((size_t)nnzb * 25), qp(5 * (size_t)nc), mup(nc), murp(nc), rhop(nc);
  c->rho_host.assign(nc, 0.0);
  std::vector<int64_t> order;
  for (int p = 0; p < nc; p++) {
    const int i = c->perm[p];
    const int64_t k0 = rowptr[i], k1 = rowptr[i + 1];
    // the row's blocks in ascending column order (the dense matrix's order)
    order.resize((size_t)(k1 - k0));
    std::iota(order.begin(), order.end(), k0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t x, int64_t y) { return colidx[x] < colidx[y]; });
    rp[p + 1] = rp[p] + (int)(k1 - k0);
    dpos[p] = -1;
    for (size_t t = 0; t < order.size(); t++) {
      const int64_t k = order[t];
      const int s = rp[p] + (int)t;
      col[s] = c->iperm[colidx[k]];
      memcpy(&W[25 * (size_t)s], &blocks[25 * k], 25 * sizeof(double));
      if (colidx[k] == i && dpos[p] < 0) dpos[p] = (int)t;
    }
    rhop[p] = 1.0 / max_eig5(&W[25 * ((size_t)rp[p] + dpos[p])]);
    c->rho_host[i] = rhop[p];
    for (int a = 0; a < 5; a++) qp[5 * (size_t)p + a] = q[5 * (size_t)i + a];
    mup[p] = mu[i];
    murp[p] = mur[i];
  }
  double s2 = 0.0;
  for (int64_t k = 0; k < 5LL * nc; k++) s2 += q[k] * q[k];
  c->norm_q = sqrt(s2);
  std::vector<double> zero(5 * (size_t)nc, 0.0);
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = upload(&c->cptr, cptr);
  if (e == cudaSuccess) e = upload(&c->rp, rp);
  if (e == cudaSuccess) e = upload(&c->col, col);
  if (e == cudaSuccess) e = upload(&c->dpos, dpos);
  if (e == cudaSuccess) e = upload(&c->W, W);
  if (e == cudaSuccess) e = upload(&c->q, qp);
  if (e == cudaSuccess) e = upload(&c->mu, mup);
  if (e == cudaSuccess) e = upload(&c->mur, murp);
  if (e == cudaSuccess) e = upload(&c->rho, rhop);
  if (e == cudaSuccess) e = upload(&c->r, zero);
  if (e == cudaSuccess) e = upload(&c->u, zero);
  {
    auto f32 = [](const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); };
    if (e == cudaSuccess) e = upload(&c->W32, f32(W));
    if (e == cudaSuccess) e = upload(&c->q32, f32(qp));
    if (e == cudaSuccess) e = upload(&c->mu32, f32(mup));
    if (e == cudaSuccess) e = upload(&c->mur32, f32(murp));
    if (e == cudaSuccess) e = upload(&c->rho32, f32(rhop));
    if (e == cudaSuccess) e = upload(&c->r32, f32(zero));
  }
  if (e != cudaSuccess) {
    free_problem(c);
    fc3dgpu_set_error("rfc3dgpu_ctx_set_problem: %s", cudaGetErrorString(e));
    return NUMERICS_ERR_UNKNOWN;
  }
  c->nc = nc;
  c->ncol = ncol;
  c->max_colour = 0;
  for (int k = 0; k < ncol; k++) c->max_colour = std::max(c->max_colour, cptr[k + 1] - cptr[k]);
  // grid: the largest colour spread over as many SMs as it fills (the local
  // Newton is bound by the FP64 pipe of each SM), smaller blocks when it
  // fills fewer SMs than the device has; all blocks resident (cooperative)
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  int threads = NT;
  while (threads > 32 && (c->max_colour + threads - 1) / threads < sms) threads /= 2;
  int per_sm = 0, per_sm32 = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rfc3d_nsgs, threads, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm32, k_rfc3d_sweeps32, threads, 0);
  const int resident = std::max(1, std::min(std::min(per_sm, per_sm32) * sms, MAX_BLOCKS));
  c->threads = threads;
  c->blocks = std::max(1, std::min((c->max_colour + threads - 1) / threads, resident));
  return 0;
}

extern "C" int rfc3dgpu_ctx_set_r(rfc3dgpu_ctx* c, const double* r) {
  if (!c || !r || c->nc == 0) return NUMERICS_ERR_INVALID_ARGUMENT;
  std::vector<double> rp(5 * (size_t)c->nc);
  for (int i = 0; i < c->nc; i++)
    for (int a = 0; a < 5; a++) rp[5 * (size_t)c->iperm[i] + a] = r[5 * (size_t)i + a];
  KR(cudaSetDevice(c->device));
  KR(cudaMemcpy(c->r, rp.data(), sizeof(double) * rp.size(), cudaMemcpyHostToDevice));
  return 0;
}

static Args args_of(const rfc3dgpu_ctx* c) {
  Args a;
  memset(&a, 0, sizeof(a));
  a.nc = c->nc;
  a.ncol = c->ncol;
  a.cptr = c->cptr;
  a.rp = c->rp;
  a.col = c->col;
  a.dpos = c->dpos;
  a.W = c->W;
  a.q = c->q;
  a.mu = c->mu;
  a.mur = c->mur;
  a.rho = c->rho;
  a.r = c->r;
  a.u = c->u;
  a.norm_q = c->norm_q;
  a.part = c->part;
  a.trace = c->trace;
  a.trace_cap = TRACE_CAP;
  a.out = c->out;
  return a;
}

static ArgsT<float> args32_of(const rfc3dgpu_ctx* c) {
  ArgsT<float> a;
  memset(&a, 0, sizeof(a));
  a.nc = c->nc;
  a.ncol = c->ncol;
  a.cptr = c->cptr;
  a.rp = c->rp;
  a.col = c->col;
  a.dpos = c->dpos;
  a.W = c->W32;
  a.q = c->q32;
  a.mu = c->mu32;
  a.mur = c->mur32;
  a.rho = c->rho32;
  a.r = c->r32;
  a.u = c->u;
  a.norm_q = c->norm_q;
  a.part = c->part;
  a.trace = c->trace;
  a.trace_cap = TRACE_CAP;
  a.out = c->out;
  return a;
}

template <typename K, typename A>
static cudaError_t launch(rfc3dgpu_ctx* c, K kernel, A& a) {
  void* params[] = {&a};
  return cudaLaunchCooperativeKernel((const void*)kernel, dim3(c->blocks), dim3(c->threads), params, 0, c->stream);
}

extern "C" int rfc3dgpu_ctx_solve(rfc3dgpu_ctx* c, double tol, int max_iter, double local_tol, int local_max_iter,
                                  int* iters, double* error, int* info, double* ms) {
  if (!c || c->nc == 0 || max_iter < 0 || local_max_iter < 0) {
    fc3dgpu_set_error("rfc3dgpu_ctx_solve: no problem or a negative budget");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  KR(cudaSetDevice(c->device));
  const int n5 = 5 * c->nc;
  KR(cudaEventRecord(c->ev[0], c->stream));
  double out[4];
  int sweeps32 = 0;
  if (c->precision == 0 && max_iter > 0) {
    // FP32 sweeps from the current reaction, then the FP64 loop from theirs
    ArgsT<float> a = args32_of(c);
    a.max_iter = max_iter;
    a.local_tol = std::max(local_tol, LOCAL_TOL32);
    a.local_max = local_max_iter;
    a.switch_tol = c->switch_tol > 0.0 ? c->switch_tol : std::max(tol, 1e-6);
    a.stall_window = c->stall;
    k_rfc3d_to_f32<<<(n5 + 255) / 256, 256, 0, c->stream>>>(n5, c->r, c->r32);
    KR(cudaGetLastError());
    KR(launch(c, k_rfc3d_sweeps32, a));
    KR(cudaMemcpyAsync(out, c->out, sizeof(out), cudaMemcpyDeviceToHost, c->stream));
    KR(cudaStreamSynchronize(c->stream));
    sweeps32 = (int)out[0];
    // a non-finite FP32 iterate is dropped: the FP64 loop starts where the
    // FP32 sweeps did
    if (out[2] == 0.0) {
      k_rfc3d_to_f64<<<(n5 + 255) / 256, 256, 0, c->stream>>>(n5, c->r32, c->r);
      KR(cudaGetLastError());
    }
  }
  Args a = args_of(c);
  a.tol = tol;
  a.max_iter = max_iter - sweeps32;
  a.local_tol = local_tol;
  a.local_max = local_max_iter;
  a.trace = c->trace + std::min(sweeps32, TRACE_CAP);
  a.trace_cap = TRACE_CAP - std::min(sweeps32, TRACE_CAP);
  KR(launch(c, k_rfc3d_nsgs, a));
  KR(cudaEventRecord(c->ev[1], c->stream));
  KR(cudaMemcpyAsync(out, c->out, sizeof(out), cudaMemcpyDeviceToHost, c->stream));
  KR(cudaStreamSynchronize(c->stream));
  float t = 0.f;
  cudaEventElapsedTime(&t, c->ev[0], c->ev[1]);
  c->sweeps32 = sweeps32;
  c->sweeps64 = (int)out[0];
  if (iters) *iters = sweeps32 + (int)out[0];
  if (error) *error = out[1];
  if (info) *info = (int)out[2];
  if (ms) *ms = t;
  c->trace_len = std::min(sweeps32 + (int)out[0], TRACE_CAP);
  return 0;
}

extern "C" int rfc3dgpu_ctx_set_precision(rfc3dgpu_ctx* c, int precision, double switch_tol, int stall_window) {
  if (!c || precision < 0 || precision > 1 || !(switch_tol >= 0.0) || stall_window < 0) {
    fc3dgpu_set_error("rfc3dgpu_ctx_set_precision: precision 0 or 1, switch_tol >= 0, stall_window >= 0");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  c->precision = precision;
  c->switch_tol = switch_tol;
  c->stall = stall_window > 0 ? stall_window : 64;
  return 0;
}

extern "C" int rfc3dgpu_ctx_last_sweeps(rfc3dgpu_ctx* c, int* sweeps32, int* sweeps64) {
  if (!c) return NUMERICS_ERR_INVALID_ARGUMENT;
  if (sweeps32) *sweeps32 = c->sweeps32;
  if (sweeps64) *sweeps64 = c->sweeps64;
  return 0;
}

extern "C" int rfc3dgpu_ctx_compute_error(rfc3dgpu_ctx* c, double norm_q, double* error) {
  if (!c || c->nc == 0 || !error) return NUMERICS_ERR_INVALID_ARGUMENT;
  KR(cudaSetDevice(c->device));
  Args a = args_of(c);
  a.norm_q = norm_q;
  KR(launch(c, k_rfc3d_error, a));
  KR(cudaMemcpyAsync(error, c->out + 1, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  KR(cudaStreamSynchronize(c->stream));
  return 0;
}

extern "C" int rfc3dgpu_ctx_get_r_u(rfc3dgpu_ctx* c, double* r, double* u) {
  if (!c || c->nc == 0) return NUMERICS_ERR_INVALID_ARGUMENT;
  KR(cudaSetDevice(c->device));
  std::vector<double> rp(5 * (size_t)c->nc), up(5 * (size_t)c->nc);
  KR(cudaMemcpy(rp.data(), c->r, sizeof(double) * rp.size(), cudaMemcpyDeviceToHost));
  KR(cudaMemcpy(up.data(), c->u, sizeof(double) * up.size(), cudaMemcpyDeviceToHost));
  for (int i = 0; i < c->nc; i++)
    for (int a = 0; a < 5; a++) {
      const size_t p = 5 * (size_t)c->iperm[i] + a;
      if (r) r[5 * (size_t)i + a] = rp[p];
      if (u) u[5 * (size_t)i + a] = up[p];
    }
  return 0;
}

extern "C" int rfc3dgpu_ctx_colours(rfc3dgpu_ctx* c, int32_t* colour) {
  if (!c || c->nc == 0) return NUMERICS_ERR_INVALID_ARGUMENT;
  if (colour) memcpy(colour, c->colour.data(), sizeof(int32_t) * c->nc);
  return c->ncol;
}

extern "C" int rfc3dgpu_ctx_rho(rfc3dgpu_ctx* c, double* rho) {
  if (!c || c->nc == 0 || !rho) return NUMERICS_ERR_INVALID_ARGUMENT;
  memcpy(rho, c->rho_host.data(), sizeof(double) * c->nc);
  return 0;
}

extern "C" int rfc3dgpu_ctx_trace(rfc3dgpu_ctx* c, double* out, int cap) {
  if (!c) return -1;
  const int n = std::min(cap, c->trace_len);
  if (n <= 0 || !out) return 0;
  KR(cudaSetDevice(c->device));
  KR(cudaMemcpy(out, c->trace, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return n;
}
