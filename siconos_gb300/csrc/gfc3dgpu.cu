// Global 3D friction contact on the GPU (include/gfc3dgpu.h): the
// reference's gfc3d_nsgs iteration (gfc3d_nsgs.c:124-178) and
// gfc3d_compute_error (gfc3d_compute_error.c:38-160) in one cooperative
// launch per solve.
//
// Layout (built on the host from the caller's CSR, once per problem):
//  * degree-of-freedom slabs: 32 rows of H (and of M) per slab, slot-major
//    (value and column of slot k of row lane at [(off[s] + k) * 32 + lane]),
//    each row's entries in ascending column order, padded with zero values
//    whose column points at a zero entry past the end of the vector;
//  * contact slabs: 32 contacts per slab, slot k holding one degree of
//    freedom j (ascending) and the three values H[j, 3c + 0..2] (zeros where
//    a component's row of H^T has no entry), so u = b + H^T v is three row
//    sums over shared columns;
//  * M^-1: LU factors of each connected component of M's pattern (column
//    major, local pivot rows), factorised on the device; when every
//    component is one degree of freedom the solve is t / M_ii, fused into
//    the row products.
//
// One iteration k:
//   phase A (degree-of-freedom rows)  t = q + H r_{k-1};  [diagonal M:
//       v_k = t / M_ii]  and the error terms of iteration k - 1: H r_{k-1}
//       and M v_{k-1} (gfc3d_compute_error.c:87-109 of r_{k-1}, v_{k-1});
//   grid barrier; the stop decision on iteration k - 1's error;
//   phase B (components, general M)  v_k = LU solve of t; grid barrier;
//   phase C (contacts)  u_k = b + H^T v_k, r_k = proj(r_{k-1} - (u_N + mu
//       |u_T|, u_T)), the complementarity terms of (r_k, u_k); grid barrier.
// The error of iteration k is thus known after phase A of iteration k + 1;
// a stop leaves r_k, u_k and v_k (v double-buffered) as the reference's loop
// leaves them.  Every product and update follows the reference's operation
// order (row sums from +0.0 in column order, then added to q or b; the
// projection as projectionOnCone), compiled without FMA contraction, so the
// iterates are the reference's bit for bit; the norms are fixed-order block
// and grid sums.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "fc3dgpu_sweep.cuh"
#include "gfc3dgpu.h"

extern "C" void fc3dgpu_set_error(const char* fmt, ...);

namespace gfc3dgpu {

using fc3dgpu::grid_barrier;
using fc3dgpu::project_cone;

constexpr int NT = 512;            // threads per block
constexpr int NW = NT / 32;
constexpr int GRID_MAX = 1024;     // blocks at most
constexpr int TRACE_CAP = 1 << 16;
constexpr int SMALL_COMPONENT = 8; // components up to this size: one thread each, else one warp
constexpr unsigned long long DEFAULT_SPIN = 1ull << 22;

struct Args {
  long long n;
  int nc, m;
  // degree-of-freedom slabs: H rows and M rows
  int nslab_d;
  const long long* hoff;
  const int* hns;
  const int* hcol;
  const double* hval;
  const long long* moff;
  const int* mns;
  const int* mcol;
  const double* mval;
  const double* q;
  const double* mdiag;  // diagonal of M when every component is one dof, else null
  // components of M (general M)
  int ncomp;
  const int* cptr;
  const int* cdof;
  const long long* luoff;
  const double* lu;
  const int* piv;
  int small;  // every component has at most SMALL_COMPONENT dofs
  // contact slabs: H^T rows
  int nslab_c;
  const long long* toff;
  const int* tns;
  const int* tcol;
  const double* tval;
  const double* b;
  const double* mu;
  double* r;     // m + 1 (r[m] = 0)
  double* u;     // m
  double* v0;    // n + 1 each (v[n] = 0): v of the odd iterations in v1, even in v0
  double* v1;
  double* t;     // n
  // solve
  double tol;
  int max_iter, freq, mode;  // mode 0 solve, 1 error of (r, v0) only, 2 v0 = M^-1 q only
  double norm_q;
  unsigned* flags;
  double* part;  // [2][GRID_MAX][8]
  int* status;
  unsigned long long spin_limit;
  double* trace;
  int trace_cap;
  double* out;  // iterations, error, info, buffer of the result's v
};

// Sum of N values over the block in a fixed order, written to out[0..N).
template <int N>
__device__ __forceinline__ void bsum(double v[N], double* out) {
  __shared__ double sh[NW][N];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < N; i++) {
    double x = v[i];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sh[w][i] = x;
  }
  __syncthreads();
  if (threadIdx.x < N) {
    double s = 0.0;
    for (int k = 0; k < NW; k++) s += sh[k][threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

// Slot i of every block's partials (stride 8) summed in a fixed order.
template <int N>
__device__ __forceinline__ void gsum(const double* part, int slot, double out[N]) {
  __shared__ double res[8];
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
#pragma unroll
    for (int i = 0; i < N; i++) {
      double s = 0.0;
      for (int bl = lane; bl < (int)gridDim.x; bl += 32) s += __ldcg(&part[bl * 8 + slot + i]);
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) res[i] = s;
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < N; i++) out[i] = res[i];
  __syncthreads();
}

// acc + a b: two roundings as the reference computes it, or (FAST, the
// opt-in fused mode) one fused multiply-add.  The translation unit is
// compiled without FMA contraction, so the first form stays unfused.
template <bool FAST>
__device__ __forceinline__ double madd(double acc, double a, double b) {
  if (FAST) return fma(a, b, acc);
  return acc + a * b;
}

// Rank of the calling warp for the grid-stride slab loops: consecutive ranks
// go to different blocks, so the slabs left over after equal shares fall
// one to a block (blocks spread over the SMs) rather than all to the first
// blocks' SMs.
__device__ __forceinline__ int warp_rank() { return (int)((threadIdx.x >> 5) * gridDim.x + blockIdx.x); }

__device__ __forceinline__ double* part_of(const Args& a, int parity) {
  return a.part + (size_t)parity * GRID_MAX * 8;
}

// Phase A over the degree-of-freedom slabs (one warp per slab).  With
// `err`, the error terms of (r, vprev) go to e[0..2] (|H r|^2, |M v|^2,
// |q + H r - M v|^2); vcur receives t / M_ii for a diagonal M (when non
// null), else t is stored.  no_h: t = q (no contact).
template <bool FAST>
__device__ __forceinline__ void phase_a(const Args& a, bool err, const double* vprev, double* vcur, bool store,
                                        bool no_h, double e[3]) {
  const int lane = threadIdx.x & 31;
  const int gw = warp_rank(), tw = (gridDim.x * NT) >> 5;
  for (int s = gw; s < a.nslab_d; s += tw) {
    const long long i = (long long)s * 32 + lane;
    const bool row = i < a.n;
    double sh = 0.0;
    if (!no_h) {
      const long long o = a.hoff[s];
      const int ns = a.hns[s];
      int k = 0;
      for (; k + 4 <= ns; k += 4) {
        double hv[4], rv[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const size_t p = (size_t)(o + k + j) * 32 + lane;
          hv[j] = __ldg(&a.hval[p]);
          rv[j] = __ldcg(&a.r[__ldg(&a.hcol[p])]);
        }
#pragma unroll
        for (int j = 0; j < 4; j++) sh = madd<FAST>(sh, hv[j], rv[j]);
      }
      for (; k < ns; k++) {
        const size_t p = (size_t)(o + k) * 32 + lane;
        sh = madd<FAST>(sh, __ldg(&a.hval[p]), __ldcg(&a.r[__ldg(&a.hcol[p])]));
      }
    }
    if (!row) continue;
    const double qi = __ldg(&a.q[i]);
    // dgemv with beta 1: 1.0 * q + 1.0 * s (the loop), daxpy q + 1.0 * tmp
    // (the error): both q + s
    const double ti = no_h ? qi : qi + 1.0 * sh;
    if (err) {
      const long long o = a.moff[s];
      const int ns = a.mns[s];
      double sm = 0.0;
      for (int k = 0; k < ns; k++) {
        const size_t p = (size_t)(o + k) * 32 + lane;
        sm = madd<FAST>(sm, __ldg(&a.mval[p]), __ldcg(&vprev[__ldg(&a.mcol[p])]));
      }
      const double hr = 0.0 + 1.0 * sh;    // NM_gemv(1.0, H, r, 0.0, tmp)
      const double mv = 0.0 + -1.0 * sm;   // NM_gemv(-1.0, M, v, 0.0, tmp)
      const double t1 = ti + 1.0 * mv;     // tmp_1 += 1.0 * tmp
      e[0] += hr * hr;
      e[1] += mv * mv;
      e[2] += t1 * t1;
    }
    if (!store) continue;
    if (vcur)
      vcur[i] = ti / __ldg(&a.mdiag[i]);
    else
      a.t[i] = ti;
  }
}

// Phase B: v = M^-1 t by the components' LU factors (gfc3d_oracle.c's
// lu_solve order: row swaps in order, forward substitution with
// subtractions in ascending column order, back substitution in descending
// order, then the division).  Small components: one thread each; larger:
// one warp, column-oriented (every element still receives its
// subtractions in the same order).
__device__ __forceinline__ void phase_b(const Args& a, double* v) {
  double* y = a.t;  // solved in place through the component's dof list
  if (a.small) {
    for (int c = blockIdx.x * NT + threadIdx.x; c < a.ncomp; c += gridDim.x * NT) {
      const int o = a.cptr[c], sz = a.cptr[c + 1] - o;
      const double* A = a.lu + a.luoff[c];
      double x[SMALL_COMPONENT];
      for (int i = 0; i < sz && i < SMALL_COMPONENT; i++) x[i] = __ldcg(&y[a.cdof[o + i]]);
      for (int i = 0; i < sz; i++) {
        const int p = a.piv[o + i];
        if (p != i) {
          const double tmp = x[i];
          x[i] = x[p];
          x[p] = tmp;
        }
      }
      for (int i = 0; i < sz; i++) {
        double w = x[i];
        for (int k = 0; k < i; k++) w = w - A[k * sz + i] * x[k];
        x[i] = w;
      }
      for (int i = sz - 1; i >= 0; i--) {
        double w = x[i];
        for (int k = sz - 1; k > i; k--) w = w - A[k * sz + i] * x[k];
        x[i] = w / A[i * sz + i];
      }
      for (int i = 0; i < sz; i++) v[a.cdof[o + i]] = x[i];
    }
    return;
  }
  const int lane = threadIdx.x & 31;
  const int gw = warp_rank(), tw = (gridDim.x * NT) >> 5;
  for (int c = gw; c < a.ncomp; c += tw) {
    const int o = a.cptr[c], sz = a.cptr[c + 1] - o;
    const double* A = a.lu + a.luoff[c];
    const int* d = a.cdof + o;
    if (lane == 0)
      for (int i = 0; i < sz; i++) {
        const int p = a.piv[o + i];
        if (p != i) {
          const double tmp = __ldcg(&y[d[i]]);
          y[d[i]] = __ldcg(&y[d[p]]);
          y[d[p]] = tmp;
        }
      }
    __syncwarp();
    for (int k = 0; k < sz; k++) {
      const double yk = __ldcg(&y[d[k]]);
      for (int i = k + 1 + lane; i < sz; i += 32) y[d[i]] = __ldcg(&y[d[i]]) - A[k * sz + i] * yk;
      __syncwarp();
    }
    for (int k = sz - 1; k >= 0; k--) {
      double yk = 0.0;
      if (lane == 0) {
        yk = __ldcg(&y[d[k]]) / A[k * sz + k];
        y[d[k]] = yk;
      }
      yk = __shfl_sync(0xffffffffu, yk, 0);
      for (int i = lane; i < k; i += 32) y[d[i]] = __ldcg(&y[d[i]]) - A[k * sz + i] * yk;
      __syncwarp();
    }
    for (int i = lane; i < sz; i += 32) v[d[i]] = __ldcg(&y[d[i]]);
  }
}

// fc3d_unitary_compute_and_add_error (fc3d_compute_error.c:42-56)
__device__ __forceinline__ double unitary_error(const double r[3], const double u[3], double mu) {
  double w[3];
  w[0] = r[0] - u[0] - mu * sqrt(u[1] * u[1] + u[2] * u[2]);
  w[1] = r[1] - u[1];
  w[2] = r[2] - u[2];
  project_cone<double>(w, mu);
  w[0] = r[0] - w[0];
  w[1] = r[1] - w[1];
  w[2] = r[2] - w[2];
  return w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
}

// Phase C over the contact slabs (one warp per slab): u = b + H^T v, the
// projected update of r (gfc3d_nsgs.c:150-165) when `update`, and the
// error terms e[0..2] (|u|^2, |r|^2, complementarity) of the result.
template <bool FAST>
__device__ __forceinline__ void phase_c(const Args& a, const double* v, bool update, double e[3]) {
  const int lane = threadIdx.x & 31;
  const int gw = warp_rank(), tw = (gridDim.x * NT) >> 5;
  for (int s = gw; s < a.nslab_c; s += tw) {
    const int c = s * 32 + lane;
    const long long o = a.toff[s];
    const int ns = a.tns[s];
    double acc[3] = {0.0, 0.0, 0.0};
    int k = 0;
    for (; k + 4 <= ns; k += 4) {
      double vv[4], tv[4][3];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const size_t p = (size_t)(o + k + j) * 32 + lane;
        vv[j] = __ldcg(&v[__ldg(&a.tcol[p])]);
        const size_t pv = (size_t)(o + k + j) * 96 + lane;
        tv[j][0] = __ldg(&a.tval[pv]);
        tv[j][1] = __ldg(&a.tval[pv + 32]);
        tv[j][2] = __ldg(&a.tval[pv + 64]);
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        acc[0] = madd<FAST>(acc[0], tv[j][0], vv[j]);
        acc[1] = madd<FAST>(acc[1], tv[j][1], vv[j]);
        acc[2] = madd<FAST>(acc[2], tv[j][2], vv[j]);
      }
    }
    for (; k < ns; k++) {
      const size_t p = (size_t)(o + k) * 32 + lane;
      const double vj = __ldcg(&v[__ldg(&a.tcol[p])]);
      const size_t pv = (size_t)(o + k) * 96 + lane;
      acc[0] = madd<FAST>(acc[0], __ldg(&a.tval[pv]), vj);
      acc[1] = madd<FAST>(acc[1], __ldg(&a.tval[pv + 32]), vj);
      acc[2] = madd<FAST>(acc[2], __ldg(&a.tval[pv + 64]), vj);
    }
    if (c >= a.nc) continue;
    double u[3], r[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      u[d] = 1.0 * __ldg(&a.b[3 * c + d]) + 1.0 * acc[d];  // dgemv^T with beta 1
      r[d] = __ldcg(&a.r[3 * c + d]);
    }
    const double mu = __ldg(&a.mu[c]);
    if (update) {
      const double normUT = sqrt(u[1] * u[1] + u[2] * u[2]);
      const double an = 1.0;
      r[0] -= an * (u[0] + mu * normUT);
      r[1] -= an * u[1];
      r[2] -= an * u[2];
      project_cone<double>(r, mu);
#pragma unroll
      for (int d = 0; d < 3; d++) a.r[3 * c + d] = r[d];
    }
#pragma unroll
    for (int d = 0; d < 3; d++) a.u[3 * c + d] = u[d];
    e[0] += u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    e[1] += r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    e[2] += unitary_error(r, u, mu);
  }
}

// gfc3d_compute_error from the grid sums of phase A (slot 0-2) and phase C
// (slot 3-5).
__device__ __forceinline__ double error_of(const Args& a, const double sa[3], const double sc[3]) {
  const double min_rel = sqrt(DBL_EPSILON);
  const double norm_hr = sqrt(sa[0]), norm_mv = sqrt(sa[1]);
  const double rel = fmax(a.norm_q, fmax(norm_mv, norm_hr));
  double err = sqrt(sa[2]);
  if (fabs(rel) > min_rel) err = err / rel;
  const double norm_u = sqrt(sc[0]), norm_r = sqrt(sc[1]);
  double ec = sqrt(sc[2]);
  const double rel2 = fmax(norm_u, norm_r);
  if (fabs(rel2) > min_rel) ec = ec / rel2;
  return err + ec;
}

template <bool FAST>
__global__ void __launch_bounds__(NT) k_gfc3d(Args a) {
  unsigned epoch = 0;
  const bool diag = a.mdiag != nullptr;
  double* vb[2] = {a.v0, a.v1};
  if (a.mode == 2) {
    // v = M^-1 q (gfc3d_driver's no-contact case)
    double e[3] = {0, 0, 0};
    phase_a<FAST>(a, false, nullptr, diag ? a.v0 : nullptr, true, true, e);
    if (!diag) {
      if (!grid_barrier(a.flags, epoch, a.spin_limit, a.status)) return;
      phase_b(a, a.v0);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.out[0] = 0;
      a.out[1] = 0.0;
      a.out[2] = 0;
      a.out[3] = 0;
    }
    return;
  }
  if (a.mode == 1) {
    // the error of (r, v0) with u = b + H^T v0 (max_iter 0, or an error
    // evaluation alone)
    double ec[3] = {0, 0, 0}, ea[3] = {0, 0, 0};
    phase_c<FAST>(a, a.v0, false, ec);
    bsum<3>(ec, part_of(a, 0) + blockIdx.x * 8 + 3);
    phase_a<FAST>(a, true, a.v0, nullptr, false, false, ea);
    bsum<3>(ea, part_of(a, 0) + blockIdx.x * 8);
    if (!grid_barrier(a.flags, epoch, a.spin_limit, a.status)) return;
    double sa[3], sc[3];
    gsum<3>(part_of(a, 0), 0, sa);
    gsum<3>(part_of(a, 0), 3, sc);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.out[0] = 0;
      a.out[1] = error_of(a, sa, sc);
      a.out[2] = -1;
      a.out[3] = 0;
    }
    return;
  }
  double eff = 1.0;  // the error the reference's loop holds (1.0 before any evaluation)
  int k = 0;
  for (;;) {
    k++;
    const int cur = k & 1, prev = cur ^ 1;
    // phase A of iteration k, with the error terms of iteration k - 1
    double ea[3] = {0, 0, 0};
    const bool final_only = k > a.max_iter;  // the error of the last iterate alone
    phase_a<FAST>(a, k >= 2, vb[prev], diag ? vb[cur] : nullptr, !final_only, false, ea);
    bsum<3>(ea, part_of(a, cur) + blockIdx.x * 8);
    if (!grid_barrier(a.flags, epoch, a.spin_limit, a.status)) return;
    if (k >= 2) {
      double sa[3], sc[3];
      gsum<3>(part_of(a, cur), 0, sa);
      gsum<3>(part_of(a, prev), 3, sc);
      const int it = k - 1;
      const double err = error_of(a, sa, sc);
      if (a.freq <= 0 || it % a.freq == 0) eff = err;
      if (a.trace && it - 1 < a.trace_cap && blockIdx.x == 0 && threadIdx.x == 0) a.trace[it - 1] = eff;
      const bool conv = eff < a.tol;
      if (conv || it >= a.max_iter) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
          a.out[0] = it;
          // at the budget the reference evaluates the error once more
          a.out[1] = it >= a.max_iter ? err : eff;
          a.out[2] = conv ? 0 : 1;
          a.out[3] = prev;
        }
        return;
      }
    }
    if (!diag) {
      phase_b(a, vb[cur]);
      if (!grid_barrier(a.flags, epoch, a.spin_limit, a.status)) return;
    }
    double ec[3] = {0, 0, 0};
    phase_c<FAST>(a, vb[cur], true, ec);
    bsum<3>(ec, part_of(a, cur) + blockIdx.x * 8 + 3);
    if (!grid_barrier(a.flags, epoch, a.spin_limit, a.status)) return;
  }
}

// Scatter M's entries into the components' dense blocks (one thread per
// row), then factorise each block (one warp per component): unblocked LU,
// first largest pivot, multipliers by division, the update of every
// element in ascending pivot order (gfc3d_oracle.c's factorise).
__global__ void k_scatter_m(long long n, const long long* mp, const int* mi, const double* mx, const int* comp_of,
                            const int* local, const int* cptr, const long long* luoff, double* lu) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = comp_of[i];
  const int sz = cptr[c + 1] - cptr[c];
  double* A = lu + luoff[c];
  for (long long k = mp[i]; k < mp[i + 1]; k++) A[(size_t)local[mi[k]] * sz + local[i]] = mx[k];
}

__global__ void k_factor(int ncomp, const int* cptr, const long long* luoff, double* lu, int* piv, int* singular) {
  const int lane = threadIdx.x & 31;
  const int c = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (c >= ncomp) return;
  const int o = cptr[c], sz = cptr[c + 1] - o;
  double* A = lu + luoff[c];
  for (int j = 0; j < sz; j++) {
    // first largest |A[i, j]|, i >= j
    double best = -1.0;
    int p = j;
    for (int i = j + lane; i < sz; i += 32) {
      const double x = fabs(A[(size_t)j * sz + i]);
      if (x > best) {
        best = x;
        p = i;
      }
    }
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, off);
      const int op = __shfl_xor_sync(0xffffffffu, p, off);
      if (ob > best || (ob == best && op < p)) {
        best = ob;
        p = op;
      }
    }
    if (lane == 0) piv[o + j] = p;
    if (A[(size_t)j * sz + p] == 0.0) {
      if (lane == 0) atomicOr(singular, 1);
      __syncwarp();
      continue;
    }
    if (p != j)
      for (int k = lane; k < sz; k += 32) {
        const double tmp = A[(size_t)k * sz + j];
        A[(size_t)k * sz + j] = A[(size_t)k * sz + p];
        A[(size_t)k * sz + p] = tmp;
      }
    __syncwarp();
    const double pj = A[(size_t)j * sz + j];
    for (int i = j + 1 + lane; i < sz; i += 32) A[(size_t)j * sz + i] = A[(size_t)j * sz + i] / pj;
    __syncwarp();
    for (int k = j + 1; k < sz; k++) {
      const double ukj = A[(size_t)k * sz + j];
      for (int i = j + 1 + lane; i < sz; i += 32)
        A[(size_t)k * sz + i] = A[(size_t)k * sz + i] - A[(size_t)j * sz + i] * ukj;
    }
    __syncwarp();
  }
}

}  // namespace gfc3dgpu

// ---------------------------------------------------------------------------
// Context (C-ABI)
// ---------------------------------------------------------------------------
using namespace gfc3dgpu;

struct gfc3dgpu_ctx {
  int device = 0;
  int sms = 0;
  int grid = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  unsigned long long spin = DEFAULT_SPIN;
  int fast = 0;  // 1: fused multiply-adds in the products (opt-in)
  long long n = 0;
  int nc = 0;
  bool ready = false;
  bool diag = false;
  int ncomp = 0, maxcomp = 0;
  double norm_q = 0.0;
  double bytes_iter = 0.0;
  int nslab_d = 0, nslab_c = 0;
  // device arrays
  long long *hoff = nullptr, *moff = nullptr, *toff = nullptr, *luoff = nullptr;
  int *hns = nullptr, *hcol = nullptr, *mns = nullptr, *mcol = nullptr, *tns = nullptr, *tcol = nullptr;
  int *cptr = nullptr, *cdof = nullptr, *piv = nullptr;
  double *hval = nullptr, *mval = nullptr, *tval = nullptr, *q = nullptr, *mdiag = nullptr, *lu = nullptr;
  double *b = nullptr, *mu = nullptr, *r = nullptr, *u = nullptr, *v[2] = {nullptr, nullptr}, *t = nullptr;
  unsigned* flags = nullptr;
  double *part = nullptr, *trace = nullptr, *out = nullptr;
  int* status = nullptr;
  int vcur = 0;  // buffer holding the current global velocity
  int trace_len = 0;
};

#define G2(x)                                                                             \
  do {                                                                                    \
    cudaError_t e_ = (x);                                                                 \
    if (e_ != cudaSuccess) {                                                              \
      fc3dgpu_set_error("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
      return NUMERICS_ERR_UNKNOWN;                                                        \
    }                                                                                     \
  } while (0)

static void free_problem(gfc3dgpu_ctx* c) {
  void* ptrs[] = {c->hoff, c->moff, c->toff, c->luoff, c->hns, c->hcol, c->mns, c->mcol, c->tns, c->tcol,
                  c->cptr, c->cdof, c->piv, c->hval, c->mval, c->tval, c->q, c->mdiag, c->lu, c->b,
                  c->mu, c->r, c->u, c->v[0], c->v[1], c->t};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  c->hoff = c->moff = c->toff = c->luoff = nullptr;
  c->hns = c->hcol = c->mns = c->mcol = c->tns = c->tcol = c->cptr = c->cdof = c->piv = nullptr;
  c->hval = c->mval = c->tval = c->q = c->mdiag = c->lu = c->b = c->mu = c->r = c->u = c->t = nullptr;
  c->v[0] = c->v[1] = nullptr;
  c->ready = false;
  c->n = 0;
  c->nc = 0;
}

extern "C" void gfc3dgpu_ctx_destroy(gfc3dgpu_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  free_problem(c);
  void* ptrs[] = {c->flags, c->part, c->trace, c->out, c->status};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" gfc3dgpu_ctx* gfc3dgpu_ctx_create(int device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    fc3dgpu_set_error("gfc3dgpu_ctx_create: no CUDA device %d", device);
    return nullptr;
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    fc3dgpu_set_error("gfc3dgpu_ctx_create: cudaSetDevice(%d) failed", device);
    return nullptr;
  }
  gfc3dgpu_ctx* c = new gfc3dgpu_ctx();
  c->device = device;
  int coop = 0;
  bool ok = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device) == cudaSuccess &&
            cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) == cudaSuccess && coop &&
            cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreate(&c->ev[0]) == cudaSuccess && cudaEventCreate(&c->ev[1]) == cudaSuccess &&
            cudaMalloc(&c->flags, sizeof(unsigned) * GRID_MAX * FC3D_FLAG_STRIDE) == cudaSuccess &&
            cudaMalloc(&c->part, sizeof(double) * 2 * GRID_MAX * 8) == cudaSuccess &&
            cudaMalloc(&c->trace, sizeof(double) * TRACE_CAP) == cudaSuccess &&
            cudaMalloc(&c->out, sizeof(double) * 8) == cudaSuccess &&
            cudaMalloc(&c->status, sizeof(int)) == cudaSuccess;
  if (!ok) {
    fc3dgpu_set_error("gfc3dgpu_ctx_create: set-up failed (%s)", cudaGetErrorString(cudaGetLastError()));
    gfc3dgpu_ctx_destroy(c);
    return nullptr;
  }
  int per_sm = 0;
  int per_sm_fast = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gfc3d<false>, NT, 0) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_fast, k_gfc3d<true>, NT, 0) != cudaSuccess ||
      std::min(per_sm, per_sm_fast) < 1) {
    fc3dgpu_set_error("gfc3dgpu_ctx_create: the solve kernel does not fit an SM");
    gfc3dgpu_ctx_destroy(c);
    return nullptr;
  }
  c->grid = std::min(GRID_MAX, c->sms * std::min(std::min(per_sm, per_sm_fast), 2));
  return c;
}

template <typename T>
static cudaError_t put(T** d, const std::vector<T>& h) {
  cudaError_t e = cudaMalloc((void**)d, sizeof(T) * std::max<size_t>(h.size(), 1));
  if (e != cudaSuccess) return e;
  if (h.empty()) return cudaSuccess;
  return cudaMemcpy(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
}

// Rows of a CSR matrix as 32-row slot-major slabs; padding gets value 0 and
// column `pad`.
static void slabs_of(long long rows, const int64_t* p, const int64_t* ix, const double* x, int pad,
                     std::vector<long long>& off, std::vector<int>& ns, std::vector<int>& col,
                     std::vector<double>& val, double* bytes) {
  const long long nslab = (rows + 31) / 32;
  off.assign(nslab + 1, 0);
  ns.assign(std::max<long long>(nslab, 1), 0);
  for (long long s = 0; s < nslab; s++) {
    long long mx = 0;
    for (long long i = s * 32; i < std::min(rows, s * 32 + 32); i++) mx = std::max<long long>(mx, p[i + 1] - p[i]);
    ns[s] = (int)mx;
    off[s + 1] = off[s] + mx;
  }
  col.assign((size_t)off[nslab] * 32, pad);
  val.assign((size_t)off[nslab] * 32, 0.0);
  for (long long s = 0; s < nslab; s++)
    for (int l = 0; l < 32; l++) {
      const long long i = s * 32 + l;
      if (i >= rows) continue;
      for (long long k = p[i]; k < p[i + 1]; k++) {
        const size_t d = (size_t)(off[s] + (k - p[i])) * 32 + l;
        col[d] = (int)ix[k];
        val[d] = x[k];
      }
    }
  *bytes += (double)p[rows] * 12.0;
}

extern "C" int gfc3dgpu_ctx_set_problem(gfc3dgpu_ctx* c, int64_t n, int nc, const int64_t* Mp, const int64_t* Mi,
                                        const double* Mx, const int64_t* Hp, const int64_t* Hi, const double* Hx,
                                        const double* q, const double* b, const double* mu) {
  if (!c || n < 1 || nc < 0 || !Mp || !Mi || !Mx || !q || (nc > 0 && (!Hp || !Hi || !Hx || !b || !mu))) {
    fc3dgpu_set_error("gfc3dgpu_ctx_set_problem: invalid argument");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  const long long m = 3LL * nc;
  if (n >= (1LL << 31) - 1 || m >= (1LL << 31) - 1) {
    fc3dgpu_set_error("gfc3dgpu_ctx_set_problem: sizes beyond 32-bit indices");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  auto check_csr = [&](const int64_t* p, const int64_t* ix, long long rows, long long cols, const char* name) {
    if (p[0] != 0) return false;
    for (long long i = 0; i < rows; i++) {
      if (p[i + 1] < p[i]) return false;
      for (long long k = p[i]; k < p[i + 1]; k++)
        if (ix[k] < 0 || ix[k] >= cols || (k > p[i] && ix[k] <= ix[k - 1])) {
          fc3dgpu_set_error("gfc3dgpu_ctx_set_problem: %s row %lld: column %lld out of range or not ascending", name,
                            i, (long long)ix[k]);
          return false;
        }
    }
    return true;
  };
  if (!check_csr(Mp, Mi, n, n, "M") || (nc > 0 && !check_csr(Hp, Hi, n, m, "H"))) {
    if (!strstr(fc3dgpu_last_error(), "row")) fc3dgpu_set_error("gfc3dgpu_ctx_set_problem: bad row pointers");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  for (int i = 0; i < nc; i++)
    if (!(mu[i] >= 0.0)) {
      fc3dgpu_set_error("gfc3dgpu_ctx_set_problem: mu[%d] = %g is not a friction coefficient", i, mu[i]);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
  // components of M's pattern, numbered by their smallest dof
  std::vector<long long> par(n);
  std::iota(par.begin(), par.end(), 0LL);
  auto find = [&](long long i) {
    while (par[i] != i) {
      par[i] = par[par[i]];
      i = par[i];
    }
    return i;
  };
  for (long long i = 0; i < n; i++)
    for (long long k = Mp[i]; k < Mp[i + 1]; k++) {
      long long x = find(i), y = find(Mi[k]);
      if (x != y) par[std::max(x, y)] = std::min(x, y);
    }
  std::vector<int> comp_of(n), id(n, -1);
  int ncomp = 0;
  for (long long i = 0; i < n; i++) {
    const long long rt = find(i);
    if (id[rt] < 0) id[rt] = ncomp++;
    comp_of[i] = id[rt];
  }
  std::vector<int> cptr(ncomp + 1, 0), cdof(n), local(n);
  for (long long i = 0; i < n; i++) cptr[comp_of[i] + 1]++;
  for (int k = 0; k < ncomp; k++) cptr[k + 1] += cptr[k];
  int maxcomp = 0;
  for (int k = 0; k < ncomp; k++) maxcomp = std::max(maxcomp, cptr[k + 1] - cptr[k]);
  if (maxcomp > GFC3DGPU_MAX_COMPONENT) {
    fc3dgpu_set_error("gfc3dgpu_ctx_set_problem: a component of M couples %d degrees of freedom (at most %d)",
                      maxcomp, GFC3DGPU_MAX_COMPONENT);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  {
    std::vector<int> fill(cptr.begin(), cptr.end() - 1);
    for (long long i = 0; i < n; i++) {
      local[i] = fill[comp_of[i]] - cptr[comp_of[i]];
      cdof[fill[comp_of[i]]++] = (int)i;
    }
  }
  std::vector<long long> luoff(ncomp + 1, 0);
  for (int k = 0; k < ncomp; k++) {
    const long long s = cptr[k + 1] - cptr[k];
    luoff[k + 1] = luoff[k] + s * s;
  }
  const bool diag = maxcomp == 1;
  std::vector<double> mdiag;
  if (diag) {
    mdiag.assign(n, 0.0);
    for (long long i = 0; i < n; i++)
      for (long long k = Mp[i]; k < Mp[i + 1]; k++)
        if (Mi[k] == i) mdiag[i] = Mx[k];
  }
  // slabs
  double bytes = 0.0;
  std::vector<long long> hoff, moff, toff;
  std::vector<int> hns, hcol, mns, mcol, tns, tcol;
  std::vector<double> hval, mval, tval;
  std::vector<int64_t> zp(n + 1, 0);
  if (nc > 0)
    slabs_of(n, Hp, Hi, Hx, (int)m, hoff, hns, hcol, hval, &bytes);
  else
    slabs_of(n, zp.data(), nullptr, nullptr, 0, hoff, hns, hcol, hval, &bytes);
  double mbytes = 0.0;
  slabs_of(n, Mp, Mi, Mx, (int)n, moff, mns, mcol, mval, &mbytes);
  // H^T by contacts: per contact the union of its three columns' dofs
  const long long nslab_c = (nc + 31) / 32;
  std::vector<std::vector<std::pair<int, int>>> byc;  std::vector<int> tcnt(std::max(nc, 1), 0);
  std::vector<int64_t> Tp(m + 1, 0), Ti, Tk;
  if (nc > 0) {
    for (long long k = 0; k < Hp[n]; k++) Tp[Hi[k] + 1]++;
    for (long long j = 0; j < m; j++) Tp[j + 1] += Tp[j];
    Ti.resize(Hp[n]);
    Tk.resize(Hp[n]);
    std::vector<int64_t> f(Tp.begin(), Tp.end() - 1);
    for (long long i = 0; i < n; i++)
      for (long long k = Hp[i]; k < Hp[i + 1]; k++) {
        const int64_t d = f[Hi[k]]++;
        Ti[d] = i;
        Tk[d] = k;
      }
  }
  // per contact: merged ascending dof list of its three H^T rows
  std::vector<std::vector<int>> cdofs(std::max(nc, 1));
  for (int cc = 0; cc < nc; cc++) {
    std::vector<int>& L = cdofs[cc];
    for (int d = 0; d < 3; d++)
      for (int64_t k = Tp[3 * cc + d]; k < Tp[3 * cc + d + 1]; k++) L.push_back((int)Ti[k]);
    std::sort(L.begin(), L.end());
    L.erase(std::unique(L.begin(), L.end()), L.end());
  }
  toff.assign(nslab_c + 1, 0);
  tns.assign(std::max<long long>(nslab_c, 1), 0);
  for (long long s = 0; s < nslab_c; s++) {
    size_t mx = 0;
    for (long long cc = s * 32; cc < std::min<long long>(nc, s * 32 + 32); cc++) mx = std::max(mx, cdofs[cc].size());
    tns[s] = (int)mx;
    toff[s + 1] = toff[s] + (long long)mx;
  }
  tcol.assign((size_t)toff[nslab_c] * 32, (int)n);
  tval.assign((size_t)toff[nslab_c] * 96, 0.0);
  for (long long s = 0; s < nslab_c; s++)
    for (int l = 0; l < 32; l++) {
      const long long cc = s * 32 + l;
      if (cc >= nc) continue;
      const std::vector<int>& L = cdofs[cc];
      for (size_t k = 0; k < L.size(); k++) tcol[(size_t)(toff[s] + k) * 32 + l] = L[k];
      for (int d = 0; d < 3; d++)
        for (int64_t e = Tp[3 * cc + d]; e < Tp[3 * cc + d + 1]; e++) {
          const size_t k = std::lower_bound(L.begin(), L.end(), (int)Ti[e]) - L.begin();
          tval[(size_t)(toff[s] + k) * 96 + (size_t)d * 32 + l] = Hx[Tk[e]];
        }
      bytes += (double)L.size() * (4.0 + 24.0);
    }
  // vectors: q, M's diagonal or t, v read and written, b, r read and
  // written, u written, mu
  bytes += (double)n * (8.0 * 4) + (double)m * (8.0 * 4) + (double)nc * 8.0;
  if (!diag) bytes += (double)luoff[ncomp] * 8.0 + (double)n * 4.0;
  bytes += mbytes;

  if (cudaSetDevice(c->device) != cudaSuccess) {
    fc3dgpu_set_error("gfc3dgpu_ctx_set_problem: cudaSetDevice failed");
    return NUMERICS_ERR_UNKNOWN;
  }
  free_problem(c);
  std::vector<double> qv(q, q + n), bv(b ? b : q, b ? b + m : q), muv(mu ? mu : q, mu ? mu + nc : q);
  std::vector<double> zero_r(m + 1, 0.0), zero_v(n + 1, 0.0);
  std::vector<long long> mp64(Mp, Mp + n + 1);
  std::vector<int> mi32(Mi, Mi + Mp[n]);
  std::vector<double> mx64(Mx, Mx + Mp[n]);
  long long* d_mp = nullptr;
  int *d_mi = nullptr, *d_comp = nullptr, *d_local = nullptr;
  double* d_mx = nullptr;
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
  };
  ok(put(&c->hoff, hoff));
  ok(put(&c->hns, hns));
  ok(put(&c->hcol, hcol));
  ok(put(&c->hval, hval));
  ok(put(&c->moff, moff));
  ok(put(&c->mns, mns));
  ok(put(&c->mcol, mcol));
  ok(put(&c->mval, mval));
  ok(put(&c->toff, toff));
  ok(put(&c->tns, tns));
  ok(put(&c->tcol, tcol));
  ok(put(&c->tval, tval));
  ok(put(&c->q, qv));
  ok(put(&c->b, bv));
  ok(put(&c->mu, muv));
  ok(put(&c->r, zero_r));
  ok(put(&c->u, std::vector<double>(std::max<long long>(m, 1), 0.0)));
  ok(put(&c->v[0], zero_v));
  ok(put(&c->v[1], zero_v));
  ok(put(&c->t, std::vector<double>(n, 0.0)));
  int singular = 0;
  if (diag) {
    ok(put(&c->mdiag, mdiag));
    for (long long i = 0; i < n; i++)
      if (mdiag[i] == 0.0) singular = 1;
  } else {
    ok(put(&c->cptr, cptr));
    ok(put(&c->cdof, cdof));
    ok(put(&c->luoff, luoff));
    ok(put(&c->piv, std::vector<int>(n, 0)));
    ok(put(&c->lu, std::vector<double>(luoff[ncomp], 0.0)));
    ok(put(&d_mp, mp64));
    ok(put(&d_mi, mi32));
    ok(put(&d_mx, mx64));
    ok(put(&d_comp, comp_of));
    ok(put(&d_local, local));
    if (e == cudaSuccess) {
      ok(cudaMemset(c->status, 0, sizeof(int)));
      k_scatter_m<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, d_mp, d_mi, d_mx, d_comp, d_local,
                                                                       c->cptr, c->luoff, c->lu);
      ok(cudaGetLastError());
      k_factor<<<(unsigned)(((long long)ncomp * 32 + 255) / 256), 256, 0, c->stream>>>(ncomp, c->cptr, c->luoff,
                                                                                       c->lu, c->piv, c->status);
      ok(cudaGetLastError());
      ok(cudaMemcpyAsync(&singular, c->status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      ok(cudaStreamSynchronize(c->stream));
    }
    void* tmp[] = {d_mp, d_mi, d_mx, d_comp, d_local};
    for (void* p : tmp)
      if (p) cudaFree(p);
  }
  if (e != cudaSuccess) {
    fc3dgpu_set_error("gfc3dgpu_ctx_set_problem: %s", cudaGetErrorString(e));
    free_problem(c);
    return NUMERICS_ERR_UNKNOWN;
  }
  if (singular) {
    fc3dgpu_set_error("gfc3dgpu_ctx_set_problem: M is singular (an exactly zero pivot)");
    free_problem(c);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  c->n = n;
  c->nc = nc;
  c->diag = diag;
  c->ncomp = ncomp;
  c->maxcomp = maxcomp;
  c->nslab_d = (int)((n + 31) / 32);
  c->nslab_c = (int)nslab_c;
  double s = 0.0;
  for (long long i = 0; i < n; i++) s += q[i] * q[i];
  c->norm_q = sqrt(s);
  c->bytes_iter = bytes;
  c->vcur = 0;
  c->trace_len = 0;
  c->ready = true;
  return 0;
}

extern "C" int gfc3dgpu_ctx_set_start(gfc3dgpu_ctx* c, const double* r, const double* v) {
  if (!c || !c->ready) {
    fc3dgpu_set_error("gfc3dgpu_ctx_set_start: no problem");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  G2(cudaSetDevice(c->device));
  const long long m = 3LL * c->nc;
  if (m > 0) {
    if (r)
      G2(cudaMemcpy(c->r, r, sizeof(double) * m, cudaMemcpyHostToDevice));
    else
      G2(cudaMemset(c->r, 0, sizeof(double) * m));
  }
  c->vcur = 0;
  if (v)
    G2(cudaMemcpy(c->v[0], v, sizeof(double) * c->n, cudaMemcpyHostToDevice));
  else
    G2(cudaMemset(c->v[0], 0, sizeof(double) * c->n));
  return 0;
}

static Args args_of(gfc3dgpu_ctx* c) {
  Args a;
  memset(&a, 0, sizeof(a));
  a.n = c->n;
  a.nc = c->nc;
  a.m = 3 * c->nc;
  a.nslab_d = c->nslab_d;
  a.hoff = c->hoff;
  a.hns = c->hns;
  a.hcol = c->hcol;
  a.hval = c->hval;
  a.moff = c->moff;
  a.mns = c->mns;
  a.mcol = c->mcol;
  a.mval = c->mval;
  a.q = c->q;
  a.mdiag = c->diag ? c->mdiag : nullptr;
  a.ncomp = c->ncomp;
  a.cptr = c->cptr;
  a.cdof = c->cdof;
  a.luoff = c->luoff;
  a.lu = c->lu;
  a.piv = c->piv;
  a.small = c->maxcomp <= SMALL_COMPONENT;
  a.nslab_c = c->nslab_c;
  a.toff = c->toff;
  a.tns = c->tns;
  a.tcol = c->tcol;
  a.tval = c->tval;
  a.b = c->b;
  a.mu = c->mu;
  a.r = c->r;
  a.u = c->u;
  // the current velocity is v0 of the launch
  a.v0 = c->v[c->vcur];
  a.v1 = c->v[c->vcur ^ 1];
  a.t = c->t;
  a.norm_q = c->norm_q;
  a.flags = c->flags;
  a.part = c->part;
  a.status = c->status;
  a.spin_limit = c->spin;
  a.trace = c->trace;
  a.trace_cap = TRACE_CAP;
  a.out = c->out;
  return a;
}

static int launch(gfc3dgpu_ctx* c, Args& a, double out[4], float* ms) {
  G2(cudaMemsetAsync(c->flags, 0, sizeof(unsigned) * GRID_MAX * FC3D_FLAG_STRIDE, c->stream));
  G2(cudaMemsetAsync(c->status, 0, sizeof(int), c->stream));
  G2(cudaEventRecord(c->ev[0], c->stream));
  void* params[] = {&a};
  const void* kern = c->fast ? (const void*)k_gfc3d<true> : (const void*)k_gfc3d<false>;
  G2(cudaLaunchCooperativeKernel(kern, dim3(c->grid), dim3(NT), params, 0, c->stream));
  G2(cudaEventRecord(c->ev[1], c->stream));
  int status = 0;
  G2(cudaMemcpyAsync(out, c->out, sizeof(double) * 4, cudaMemcpyDeviceToHost, c->stream));
  G2(cudaMemcpyAsync(&status, c->status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  G2(cudaStreamSynchronize(c->stream));
  if (ms) cudaEventElapsedTime(ms, c->ev[0], c->ev[1]);
  if (status) {
    fc3dgpu_set_error("gfc3dgpu: a grid-barrier wait reached its poll limit (status %d)", status);
    return NUMERICS_ERR_UNKNOWN;
  }
  return 0;
}

extern "C" int gfc3dgpu_ctx_solve(gfc3dgpu_ctx* c, double tol, int max_iter, int freq, int* iters, double* error,
                                  int* info, double* ms) {
  if (!c || !c->ready) {
    fc3dgpu_set_error("gfc3dgpu_ctx_solve: no problem");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (max_iter < 0) {
    fc3dgpu_set_error("gfc3dgpu_ctx_solve: negative iteration budget");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  G2(cudaSetDevice(c->device));
  Args a = args_of(c);
  a.tol = tol;
  a.max_iter = max_iter;
  a.freq = freq;
  a.mode = c->nc == 0 ? 2 : (max_iter == 0 ? 1 : 0);
  double out[4] = {0, 0, 0, 0};
  float t = 0.f;
  const int rc = launch(c, a, out, &t);
  if (rc) return rc;
  // v0 of the launch is buffer c->vcur; the result lies in v0 or v1
  c->vcur ^= (int)out[3];
  if (iters) *iters = (int)out[0];
  if (error) *error = out[1];
  if (info) *info = (int)out[2];
  if (ms) *ms = t;
  c->trace_len = a.mode == 0 ? std::min((int)out[0], TRACE_CAP) : 0;
  return 0;
}

extern "C" int gfc3dgpu_ctx_compute_error(gfc3dgpu_ctx* c, double norm_q, double* error) {
  if (!c || !c->ready || c->nc == 0) {
    fc3dgpu_set_error("gfc3dgpu_ctx_compute_error: no problem with contacts");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  G2(cudaSetDevice(c->device));
  Args a = args_of(c);
  a.mode = 1;
  if (norm_q >= 0.0) a.norm_q = norm_q;
  double out[4];
  const int rc = launch(c, a, out, nullptr);
  if (rc) return rc;
  if (error) *error = out[1];
  return 0;
}

extern "C" int gfc3dgpu_ctx_get(gfc3dgpu_ctx* c, double* r, double* u, double* v) {
  if (!c || !c->ready) {
    fc3dgpu_set_error("gfc3dgpu_ctx_get: no problem");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  G2(cudaSetDevice(c->device));
  const long long m = 3LL * c->nc;
  if (r && m) G2(cudaMemcpy(r, c->r, sizeof(double) * m, cudaMemcpyDeviceToHost));
  if (u && m) G2(cudaMemcpy(u, c->u, sizeof(double) * m, cudaMemcpyDeviceToHost));
  if (v) G2(cudaMemcpy(v, c->v[c->vcur], sizeof(double) * c->n, cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int gfc3dgpu_ctx_trace(gfc3dgpu_ctx* c, double* out, int cap) {
  if (!c) return -1;
  const int n = std::min(cap, c->trace_len);
  if (n <= 0 || !out) return 0;
  G2(cudaSetDevice(c->device));
  G2(cudaMemcpy(out, c->trace, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return n;
}

extern "C" int gfc3dgpu_ctx_info(gfc3dgpu_ctx* c, int* ncomp, int* max_component, int* diagonal,
                                 double* bytes_per_iteration, int* grid) {
  if (!c || !c->ready) {
    fc3dgpu_set_error("gfc3dgpu_ctx_info: no problem");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (ncomp) *ncomp = c->ncomp;
  if (max_component) *max_component = c->maxcomp;
  if (diagonal) *diagonal = c->diag ? 1 : 0;
  if (bytes_per_iteration) *bytes_per_iteration = c->bytes_iter;
  if (grid) *grid = c->grid;
  return 0;
}

extern "C" int gfc3dgpu_ctx_set_arithmetic(gfc3dgpu_ctx* c, int fused) {
  if (!c || (fused != 0 && fused != 1)) {
    fc3dgpu_set_error("gfc3dgpu_ctx_set_arithmetic: 0 (the reference's) or 1 (fused multiply-adds)");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  c->fast = fused;
  return 0;
}

extern "C" int gfc3dgpu_ctx_spin_limit(gfc3dgpu_ctx* c, unsigned long long polls) {
  if (!c) return NUMERICS_ERR_INVALID_ARGUMENT;
  c->spin = polls ? polls : DEFAULT_SPIN;
  return 0;
}
