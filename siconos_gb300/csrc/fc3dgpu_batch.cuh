// Batched persistent NSGS: many independent FC3D problems in one launch.
//
// The problems are one block-diagonal union layout (rows permuted by
// problem, then colour, each (problem, colour) group padded to 32-row slabs).
// Each block pulls whole problems from a work queue ordered by decreasing
// size, and runs every sweep of its problem with block barriers between
// colours -- no grid-wide synchronisation at all.  Within a problem the
// arithmetic is that of the single-problem kernel (same row product, same
// local solver, same reference convergence logic with fc3d_compute_error and
// the tolerance manager), so each problem's iterates equal a solo solve's.
#pragma once
#include "fc3dgpu_batch_args.cuh"
#include "fc3dgpu_sweep.cuh"

namespace fc3dgpu {

__device__ __forceinline__ void block_reduce3(double v[3], double out[3]) {
  __shared__ double sh[FC3D_BLOCK_MAX / 32][3];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    double x = v[i];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sh[w][i] = x;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 3; i++) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k][i];
    out[i] = s;
  }
  __syncthreads();
}

template <typename Real>
__device__ __forceinline__ double scene_full_error(const SweepArgs<Real>& a, int p0, int p1, double norm_q) {
  double v[3], s[3];
  full_error_rows(a, v, p0, p1, threadIdx.x, blockDim.x);
  block_reduce3(v, s);
  double e = sqrt(s[0]);
  const double scal = fmax(norm_q, fmax(sqrt(s[2]), sqrt(s[1])));
  if (fabs(scal) > DBL_EPSILON) e /= scal;
  return e;
}

template <typename Real>
__device__ __forceinline__ void solve_scene(const BatchArgs<Real>& b, int scene, WorkList<Real>& wk) {
  const SweepArgs<Real>& a = b.base;
  const int ncol = b.scene_ncol[scene];
  const int* sptr = b.scene_sptr + (size_t)scene * (FC3D_MAX_COLOURS + 1);
  const int p0 = sptr[0] * FC3D_SLAB, p1 = sptr[ncol] * FC3D_SLAB;
  const double norm_q = b.scene_normq[scene];
  const int max_sweeps = b.scene_budget ? b.scene_budget[scene] : a.max_sweeps;
  double working = a.mode == 1 ? a.user_tol : fmax(a.user_tol, a.switch_tol), local_tol = a.local_tol;
  double incr = INFINITY, full = INFINITY, best = INFINITY;
  int sweep = 0, best_sweep = 0;
  bool converged = false;
  if (a.mode == 1 && b.scene_out_prev && b.scene_out_prev[(size_t)scene * 8 + 3] == 0.0) {
    // the FP32 iterate met the tolerance in FP32 arithmetic: FP64 check first
    full = scene_full_error(a, p0, p1, norm_q);
    if (full < a.user_tol) {
      if (threadIdx.x == 0) {
        double* o = b.scene_out + (size_t)scene * 8;
        o[0] = 0;
        o[1] = b.scene_out_prev[(size_t)scene * 8 + 1];
        o[2] = full;
        o[3] = 0;
        o[4] = working;
        o[5] = local_tol;
      }
      return;
    }
  }
  while (sweep < max_sweeps) {
    sweep++;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int c = 0; c < ncol; c++) {
      process_range_compact<Real>(a, sptr[c], sptr[c + 1], (Real)local_tol, acc[0], acc[1], wk, nullptr);
      __syncthreads();
    }
    double s[3];
    block_reduce3(acc, s);
    incr = sqrt(s[0]);
    const double nr = sqrt(s[1]);
    if (fabs(nr) > DBL_EPSILON) incr /= nr;
    bool stop = false;
    if (a.mode == 1) {
      if (incr < working) {
        full = scene_full_error(a, p0, p1, norm_q);
        if (full <= a.user_tol) {
          converged = true;
          stop = true;
        } else if (incr < 1e-15 || incr < DBL_EPSILON * 100.0) {
          local_tol = fmax(local_tol / 100.0, DBL_EPSILON * 1e-6);
        } else if (full > 0.0 && incr > 0.0) {
          double nt = (incr / full) * a.user_tol;
          const double user_min = a.user_tol * 1e-6, floor_tol = DBL_EPSILON * 1e-6;
          const double mint = user_min > floor_tol ? user_min : floor_tol;
          if (nt < mint) nt = mint;
          if (nt > 0.0 && nt < working) working = nt;
        }
        if (!(working > 0.0)) stop = true;
      }
    } else {
      if (!(incr == incr)) {
        if (threadIdx.x == 0) atomicOr(a.status, 2);
        stop = true;
      }
      if (incr < a.switch_tol) stop = true;
      if (incr < 0.99 * best) {
        best = incr;
        best_sweep = sweep;
      } else if (a.stall_window > 0 && sweep - best_sweep >= a.stall_window) {
        stop = true;
      }
      // the reference's adaptive test on this precision's iterate, against
      // max(tol, switch_tol), as in the single-problem kernel
      if (!stop && incr < working) {
        full = scene_full_error(a, p0, p1, norm_q);
        const double target = fmax(a.user_tol, a.switch_tol);
        if (full <= target) {
          converged = true;
          stop = true;
        } else if (full > 0.0 && incr > 0.0) {
          double nt = (incr / full) * target;
          const double mint = fmax(target * 1e-6, DBL_EPSILON * 1e-6);
          if (nt < mint) nt = mint;
          if (nt < working) working = nt;
        }
      }
    }
    if (stop) break;
  }
  int info = 1;
  if (a.mode == 1) {
    full = scene_full_error(a, p0, p1, norm_q);
    info = full < a.user_tol ? 0 : 1;
    if (sweep == max_sweeps && info > 0) info = -20;
  } else {
    info = converged ? 0 : 1;
  }
  if (threadIdx.x == 0) {
    double* o = b.scene_out + (size_t)scene * 8;
    o[0] = sweep;
    o[1] = incr;
    o[2] = full;
    o[3] = info;
    o[4] = working;
    o[5] = local_tol;
  }
}

template <typename Real>
__global__ void __launch_bounds__(BlockDim<Real>::value, 1) nsgs_batch_kernel(const BatchArgs<Real> b) {
  __shared__ WorkList<Real> wk;
  __shared__ int s_next;
  for (;;) {
    if (threadIdx.x == 0) s_next = atomicAdd(b.queue, 1);
    __syncthreads();
    const int k = s_next;
    __syncthreads();
    if (k >= b.nscenes) break;
    solve_scene<Real>(b, b.order[k], wk);
    __syncthreads();
  }
}

}  // namespace fc3dgpu
