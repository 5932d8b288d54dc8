// Coloured NSGS for 2D friction contact on the GPU (include/fc2dgpu.h).
//
// Layout: contacts permuted by colour (stable in contact order); per permuted
// row its blocks in the caller's order (diagonal included, at dpos), each a
// 2x2 column-major block, with the permuted column index; q, mu, r, u in
// permuted order.  One thread-block cluster per problem, or a cooperative
// grid over every SM when a colour is larger than a cluster (k_fc2d_nsgs).
// FP64 without FMA contraction, in the reference's operation order.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "fc2dgpu.h"

extern "C" void fc3dgpu_set_error(const char* fmt, ...);

namespace fc2dgpu {

namespace cg = cooperative_groups;

constexpr int NT_MAX = 512;  // threads per block at most
constexpr int CS_MAX = 16;   // blocks per cluster at most (non-portable size)
constexpr int MAXC = 128;
constexpr int TRACE_CAP = 1 << 16;
constexpr size_t REP_MAX_BYTES = 208 * 1024;  // shared-memory copy of the reactions at most
constexpr int GRID_MAX = 1024;                 // blocks of a cooperative grid at most

template <typename T>
struct Vec2;
template <>
struct Vec2<double> {
  using type = double2;
};
template <>
struct Vec2<float> {
  using type = float2;
};

// Sweep modes: the reference's error evaluations (fc2d_nsgs.c:438-448,
// :496-500) in FP64, and the FP32 phase of the mixed-precision solve.
enum Mode { FULL_FINAL = 0, LIGHT = 1, NO_EVAL = 2, FP32_PHASE = 3 };

template <typename T>
struct Args {
  int nc, ncol;
  const int* cptr;  // ncol + 1 permuted-row bounds of the colours
  const int* rp;    // nc + 1 slot pointer per permuted row
  const int* col;   // permuted column of each slot
  const int* dpos;  // offset in the row of its first diagonal block
  const T* W;       // 4 per slot
  const T* det;     // determinant of each row's diagonal block
  const T* q;
  const T* mu;
  double* r;        // the reactions (FP64, permuted order)
  T* rw;            // the sweep's copy in HBM when it is not replicated
  double* u;
  double norm_q, tol;
  int max_iter;
  int mode;
  double switch_tol;      // FP32 phase: stop below this light error
  int stall;              // FP32 phase: stop after this many sweeps without a new lowest error
  const double* before;   // out[] of the phase run before this one (or null)
  double* part;           // grid team: 2 x GRID_MAX x 4 block partial sums
  double* trace;
  double* out;  // [0] sweeps, [1] final error, [2] info, [3] last light error
};

// The blocks that share a solve.  A thread-block cluster (up to 16 SMs):
// hardware cluster barrier, partial sums exchanged through distributed
// shared memory.  A cooperative grid (every SM, for colours too large for a
// cluster): grid barrier, partial sums through a ring in global memory.
struct ClusterTeam {
  static constexpr bool grid = false;
  cg::cluster_group cl;
  __device__ ClusterTeam() : cl(cg::this_cluster()) {}
  __device__ __forceinline__ int rank() const { return (int)cl.block_rank(); }
  __device__ __forceinline__ int size() const { return (int)cl.num_blocks(); }
  // barrier between colours: the hardware cluster barrier (about 670 cycles
  // on this part), or the block barrier (about 290) for a one-block cluster
  __device__ __forceinline__ void sync() {
    if (size() == 1)
      __syncthreads();
    else
      cl.sync();
  }
  __device__ __forceinline__ void sync_all() { cl.sync(); }
};

struct GridTeam {
  static constexpr bool grid = true;
  cg::grid_group g;
  __device__ GridTeam() : g(cg::this_grid()) {}
  __device__ __forceinline__ int rank() const { return (int)blockIdx.x; }
  __device__ __forceinline__ int size() const { return (int)gridDim.x; }
  __device__ __forceinline__ void sync() {
    if (gridDim.x == 1)
      __syncthreads();
    else
      g.sync();
  }
  __device__ __forceinline__ void sync_all() { sync(); }
};

// Where the sweep keeps the reactions.  HBM: read past L1 (ld.global.cg)
// so every block sees the cluster's latest values after a cluster barrier.
// Replicated: a full copy in the shared memory of every block of the
// cluster; the owner of a contact writes its new reaction into all copies
// (distributed shared memory stores), so every read in the sweep is a local
// shared-memory load.  W and the per-contact constants are read-only and
// stay in the L1 of the block that owns the contact.
template <typename T, bool REP>
struct Reactions {
  using V = typename Vec2<T>::type;
  V* rs;  // this block's copy (REP)
  T* rw;  // HBM copy
  __device__ __forceinline__ V get(int j) const {
    if (REP) return rs[j];
    return __ldcg(reinterpret_cast<const V*>(rw) + j);
  }
  template <typename Team>
  __device__ __forceinline__ void put(int j, T x0, T x1, Team& t) const {
    V v;
    v.x = x0;
    v.y = x1;
    if constexpr (REP && !Team::grid) {
      const int cs = t.size();
      for (int k = 0; k < cs; k++) t.cl.map_shared_rank(rs, k)[j] = v;
    } else {
      __stcg(reinterpret_cast<V*>(rw) + j, v);
    }
  }
};

template <typename T, typename V>
__device__ __forceinline__ void mvp2x2(const T* a, const V v, T* y) {
  const V a01 = __ldg(reinterpret_cast<const V*>(a));
  const V a23 = __ldg(reinterpret_cast<const V*>(a) + 1);
  y[0] += a01.x * v.x;
  y[1] += a01.y * v.x;
  y[0] += a23.x * v.y;
  y[1] += a23.y * v.y;
}

// Team-wide sum of N values per thread, in a fixed order (xor-shuffle tree
// in each warp, the warps in order, then the blocks in rank order), so every
// block gets the same bits.  The barrier inside also orders every reaction
// update made before the call.  The block partials go through a two-slot
// ring (shared memory of each cluster block, or global memory for a grid): a
// block writes slot k & 1 only after the barrier of call k - 1, which every
// block passes after reading call k - 2's slot.
template <typename T>
struct Reduce {
  T part[2][4];
  T warp[NT_MAX / 32][4];
  T bcast[4];
  int calls;
};

template <int N, typename T, typename Team>
__device__ __forceinline__ void team_sum(T v[N], Reduce<T>& R, Team& team, double* gpart) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < N; i++) {
    T x = v[i];
    for (int o = 16; o >= 1; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) R.warp[w][i] = x;
  }
  __syncthreads();
  const int slot = R.calls & 1;
  double* gslot = gpart + (size_t)slot * GRID_MAX * 4;
  if (threadIdx.x == 0) {
    for (int i = 0; i < N; i++) {
      T s = 0;
      for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += R.warp[k][i];
      if constexpr (Team::grid)
        __stcg(&gslot[4 * blockIdx.x + i], (double)s);
      else
        R.part[slot][i] = s;
    }
  }
  team.sync();
  if constexpr (Team::grid) {
    // thread 0 adds the blocks' partials in order
    if (threadIdx.x == 0) {
      for (int i = 0; i < N; i++) {
        T s = 0;
        for (int b = 0; b < (int)gridDim.x; b++) s += (T)__ldcg(&gslot[4 * b + i]);
        R.bcast[i] = s;
      }
      R.calls++;
    }
  } else if (w == 0) {
    // lane k fetches block k's partials (the remote loads overlap), lane 0
    // adds them in rank order
    const int cs = team.size();
    T mine[N];
#pragma unroll
    for (int i = 0; i < N; i++) mine[i] = lane < cs ? team.cl.map_shared_rank(&R.part[slot][0], lane)[i] : T(0);
#pragma unroll
    for (int i = 0; i < N; i++) {
      T s = 0;
      for (int k = 0; k < cs; k++) s += __shfl_sync(0xffffffffu, mine[i], k);
      if (lane == 0) R.bcast[i] = s;
    }
    if (lane == 0) R.calls++;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < N; i++) v[i] = R.bcast[i];
  __syncthreads();
}

// fc2d_compute_error (fc2d_compute_error.c:40-140): u = q + W r block by
// block (per block w_i = 1.0 w_i + 1.0 (a_i0 r0 + a_i1 r1), the reference's
// 2x2 gemv), natural-map error, relative to max(|r|, |u|, |q|).  FP64 only.
template <bool REP, typename Team>
__device__ double full_error(const Args<double>& a, const Reactions<double, REP>& rx, Reduce<double>& R,
                             Team& team) {
  double v[3] = {0.0, 0.0, 0.0};
  const int g0 = team.rank() * blockDim.x + threadIdx.x, G = team.size() * blockDim.x;
  for (int p = g0; p < a.nc; p += G) {
    double w[2] = {a.q[2 * p], a.q[2 * p + 1]};
    for (int s = a.rp[p]; s < a.rp[p + 1]; s++) {
      const double* blk = a.W + 4 * (size_t)s;
      const double2 x = rx.get(a.col[s]);
      for (int i = 0; i < 2; i++) {
        double t = 0.0;
        t += blk[i] * x.x;
        t += blk[2 + i] * x.y;
        w[i] = 1.0 * w[i] + 1.0 * t;
      }
    }
    __stcg(reinterpret_cast<double2*>(a.u) + p, make_double2(w[0], w[1]));
    const double2 rr = rx.get(p);
    const double r0 = rr.x, r1 = rr.y, mu = a.mu[p];
    double t0 = r0 - w[0] - mu * fabs(w[1]);
    double t1 = r1 - w[1];
    const double normT = fabs(t1);
    if (mu * normT <= -t0) {
      t0 = 0.;
      t1 = 0.;
    } else if (normT > mu * t0) {
      t0 = (mu * normT + t0) / (mu * mu + 1.0);
      t1 = mu * t0 * (double)((t1 > 0) - (t1 < 0));
    }
    t0 = r0 - t0;
    t1 = r1 - t1;
    v[0] += t0 * t0 + t1 * t1;
    v[1] += r0 * r0 + r1 * r1;
    v[2] += w[0] * w[0] + w[1] * w[1];
  }
  team_sum<3>(v, R, team, a.part);
  double e = sqrt(v[0]);
  const double scal = fmax(sqrt(v[1]), fmax(sqrt(v[2]), a.norm_q));
  if (fabs(scal) > DBL_EPSILON) e /= scal;
  return e;
}

// fc2d_nsgs_local_solve (fc2d_nsgs.c:212-252), in the working precision
template <typename T>
__device__ __forceinline__ void local_solve(const T* W, T D, const T* q, T mu, T* P) {
  const T Wnn = W[0], Wtn = W[1], Wnt = W[2], Wtt = W[3];
  if (q[0] > 0) {
    P[0] = 0;
    P[1] = 0;
  } else {
    P[0] = -(Wtt * q[0] - Wnt * q[1]) / D;
    P[1] = -(-Wtn * q[0] + Wnn * q[1]) / D;
    const T muPn = mu * P[0];
    if (fabs(P[1]) > muPn) {
      if (P[1] + muPn < 0) {
        P[0] = -q[0] / (Wnn - mu * Wnt);
        P[1] = -mu * P[0];
      } else {
        P[0] = -q[0] / (Wnn + mu * Wnt);
        P[1] = mu * P[0];
      }
    }
  }
}

// Bring the FP64 reactions into the sweep's copy (replica or FP32 copy in
// HBM); the cluster barrier keeps other blocks from writing into a copy
// before it is filled.
template <typename T, bool REP, typename Team>
__device__ __forceinline__ Reactions<T, REP> open_reactions(const Args<T>& a, typename Vec2<T>::type* smem,
                                                            Team& team) {
  using V = typename Vec2<T>::type;
  Reactions<T, REP> rx{smem, a.rw};
  const double2* r = reinterpret_cast<const double2*>(a.r);
  if (REP) {
    for (int j = threadIdx.x; j < a.nc; j += blockDim.x) {
      const double2 x = __ldcg(r + j);
      V v;
      v.x = (T)x.x;
      v.y = (T)x.y;
      smem[j] = v;
    }
    team.sync_all();
  } else if (sizeof(T) != sizeof(double)) {
    const int g0 = team.rank() * blockDim.x + threadIdx.x, G = team.size() * blockDim.x;
    for (int j = g0; j < a.nc; j += G) {
      const double2 x = __ldcg(r + j);
      V v;
      v.x = (T)x.x;
      v.y = (T)x.y;
      __stcg(reinterpret_cast<V*>(a.rw) + j, v);
    }
    team.sync_all();
  }
  return rx;
}

// Write the sweep's copy back to the FP64 reactions (each block its own
// contacts), then hold every block until no other may still read its
// shared memory.
template <typename T, bool REP, typename Team>
__device__ __forceinline__ void close_reactions(const Args<T>& a, const Reactions<T, REP>& rx, Team& team) {
  if (REP || sizeof(T) != sizeof(double)) {
    const int g0 = team.rank() * blockDim.x + threadIdx.x, G = team.size() * blockDim.x;
    for (int p = g0; p < a.nc; p += G) {
      const typename Vec2<T>::type x = rx.get(p);
      __stcg(reinterpret_cast<double2*>(a.r) + p, make_double2((double)x.x, (double)x.y));
    }
  }
  team.sync_all();
}

// All sweeps of one problem (or of one precision phase of it) in one launch
// of one thread-block cluster or one cooperative grid (the Team).  A colour's contacts are spread over the
// cluster's threads (contact lo + g, lo + g + G, ... for global thread g of
// G: a contact always lands on the same block, so its W row stays in that
// SM's L1); the hardware cluster barrier (release / acquire) separates
// colours, the barrier of the error reduction closing the last one, and the
// convergence logic runs on the device with the same bits in every block.
// The light error's |r|^2 is summed over the new reactions as they are made
// (each contact is updated once per sweep, so it is |r|^2 after the sweep).
// A phase that follows another starts its sweep count, budget and trace
// where the previous one stopped (read from the device, no host round trip).
template <typename T, bool REP, typename Team>
__global__ void __launch_bounds__(NT_MAX, 1) k_fc2d_nsgs(const Args<T> a) {
  using V = typename Vec2<T>::type;
  extern __shared__ __align__(16) unsigned char dsm[];
  V* rsm = reinterpret_cast<V*>(dsm);
  __shared__ Reduce<T> R;
  Team team;
  if (threadIdx.x == 0) R.calls = 0;
  __syncthreads();
  const Reactions<T, REP> rx = open_reactions<T, REP>(a, rsm, team);
  const int g0 = team.rank() * blockDim.x + threadIdx.x, G = team.size() * blockDim.x;
  const bool lead = team.rank() == 0 && threadIdx.x == 0;
  const int done = a.before ? (int)a.before[0] : 0;
  const int budget = a.max_iter - done;
  T tolerance = (T)a.tol, err = (T)INFINITY, best = (T)INFINITY;
  int iter = 0, not_conv = 1, since_best = 0;
  while (iter < budget && not_conv) {
    ++iter;
    T v[2] = {0, 0};
    for (int c = 0; c < a.ncol; c++) {
      for (int p = a.cptr[c] + g0; p < a.cptr[c + 1]; p += G) {
        const V old = rx.get(p);
        T ql[2] = {a.q[2 * p], a.q[2 * p + 1]};
        const int s0 = a.rp[p], s1 = a.rp[p + 1], sd = s0 + a.dpos[p];
        // every block on the diagonal is left out (SBM_row_prod_no_diag_2x2);
        // a row of up to NB blocks has all its neighbours' reactions fetched
        // before the first product (one memory round trip, not one per
        // block), then the products run in the row's order
        constexpr int NB = sizeof(T) == sizeof(float) ? 16 : 8;
        if (s1 - s0 <= NB) {
          int cj[NB];
          V rj[NB];
#pragma unroll
          for (int k = 0; k < NB; k++)
            if (k < s1 - s0) cj[k] = a.col[s0 + k];
#pragma unroll
          for (int k = 0; k < NB; k++)
            if (k < s1 - s0 && cj[k] != p) rj[k] = rx.get(cj[k]);
#pragma unroll
          for (int k = 0; k < NB; k++)
            if (k < s1 - s0 && cj[k] != p) mvp2x2(a.W + 4 * (size_t)(s0 + k), rj[k], ql);
        } else {
          for (int s = s0; s < s1; s++) {
            const int j = a.col[s];
            if (j != p) mvp2x2(a.W + 4 * (size_t)s, rx.get(j), ql);
          }
        }
        T P[2] = {old.x, old.y};
        local_solve<T>(a.W + 4 * (size_t)sd, a.det[p], ql, a.mu[p], P);
        const T x0 = old.x - P[0], x1 = old.y - P[1];
        v[0] += x0 * x0 + x1 * x1;
        v[1] += P[0] * P[0] + P[1] * P[1];
        rx.put(p, P[0], P[1], team);
      }
      if (c + 1 < a.ncol) team.sync();
    }
    team_sum<2>(v, R, team, a.part);
    err = sqrt(v[0]);
    const T nr = sqrt(v[1]);
    if (fabs(nr) > (T)DBL_EPSILON) err /= nr;
    if (a.trace && lead && done + iter <= TRACE_CAP) a.trace[done + iter - 1] = (double)err;
    if (a.mode == FP32_PHASE) {
      if (err < best) {
        best = err;
        since_best = 0;
      } else {
        since_best++;
      }
      not_conv = !(err < (T)a.switch_tol) && since_best < a.stall;
    } else if (a.mode == LIGHT) {
      not_conv = !(err < tolerance);  // determine_convergence (fc2d_nsgs.c:147-162)
    } else if (a.mode == FULL_FINAL && err < tolerance) {
      // determine_convergence_with_full_final (fc2d_nsgs.c:187-228)
      not_conv = 0;
      if constexpr (sizeof(T) == sizeof(double)) {
        const double full = full_error<REP>(a, rx, R, team);
        if (full > a.tol) {
          tolerance = err / full * a.tol;
          not_conv = 1;
        }
      }
    }
  }
  double final_err = (double)err;
  if constexpr (sizeof(T) == sizeof(double)) {
    if (a.mode == FULL_FINAL) {
      final_err = full_error<REP>(a, rx, R, team);
      not_conv = !(final_err < a.tol);
    } else if (a.mode == NO_EVAL) {
      final_err = INFINITY;  // no branch of the sweep loop evaluates an error (fc2d_nsgs.c:438-448)
      not_conv = 1;
    }
  }
  if (lead) {
    a.out[0] = done + iter;
    a.out[1] = final_err;
    a.out[2] = not_conv;
    a.out[3] = (double)err;
  }
  close_reactions<T, REP>(a, rx, team);
}

template <bool REP, typename Team>
__global__ void __launch_bounds__(NT_MAX, 1) k_fc2d_error(const Args<double> a) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ Reduce<double> R;
  Team team;
  if (threadIdx.x == 0) R.calls = 0;
  __syncthreads();
  const Reactions<double, REP> rx = open_reactions<double, REP>(a, reinterpret_cast<double2*>(dsm), team);
  const double e = full_error<REP>(a, rx, R, team);
  if (team.rank() == 0 && threadIdx.x == 0) a.out[1] = e;
  close_reactions<double, REP>(a, rx, team);
}

}  // namespace fc2dgpu

// ---------------------------------------------------------------------------
// Context (C-ABI)
// ---------------------------------------------------------------------------
using namespace fc2dgpu;

struct fc2dgpu_ctx {
  int device = 0;
  int cs_req = 0, nt_req = 0;  // launch shape asked for (0 = automatic)
  int rep_req = 0;             // reactions: 0 automatic, 1 in HBM, 2 replicated in shared memory
  int cs = 1, nt = 128;        // launch shape of the current problem
  bool rep = false;
  bool grid = false;           // a cooperative grid of `blocks` blocks instead of a cluster
  int blocks = 1;
  int max_colour = 0;          // contacts in the largest colour
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  int nc = 0, ncol = 0;
  bool singular = false;
  double norm_q = 0.0;
  std::vector<int> perm, iperm, colour;
  int *cptr = nullptr, *rp = nullptr, *col = nullptr, *dpos = nullptr;
  double *W = nullptr, *det = nullptr, *q = nullptr, *mu = nullptr, *r = nullptr, *u = nullptr, *trace = nullptr,
         *out = nullptr, *part = nullptr;
  // FP32 copies for the first phase of a mixed-precision solve
  float *W32 = nullptr, *det32 = nullptr, *q32 = nullptr, *mu32 = nullptr, *r32 = nullptr;
  int precision = 1;          // 0 FP32 sweeps + FP64 polish, 1 FP64 sweeps only
  double switch_tol = 0.0;    // FP32 phase stops below this light error (0: max(tol, 1e-6))
  int stall = 64;             // ... or after this many sweeps without a new lowest error
  int sweeps32 = 0, sweeps64 = 0;
  int trace_len = 0;
};

#define K2(x)                                                                             \
  do {                                                                                    \
    cudaError_t e_ = (x);                                                                 \
    if (e_ != cudaSuccess) {                                                              \
      fc3dgpu_set_error("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
      return NUMERICS_ERR_UNKNOWN;                                                        \
    }                                                                                     \
  } while (0)

static void choose_shape(fc2dgpu_ctx* c);

static void free_problem(fc2dgpu_ctx* c) {
  void* ptrs[] = {c->cptr, c->rp, c->col, c->dpos, c->W, c->det, c->q, c->mu, c->r, c->u,
                  c->W32, c->det32, c->q32, c->mu32, c->r32};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  c->cptr = c->rp = c->col = c->dpos = nullptr;
  c->W = c->det = c->q = c->mu = c->r = c->u = nullptr;
  c->W32 = c->det32 = c->q32 = c->mu32 = c->r32 = nullptr;
  c->nc = 0;
}

extern "C" void fc2dgpu_ctx_destroy(fc2dgpu_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  free_problem(c);
  if (c->trace) cudaFree(c->trace);
  if (c->out) cudaFree(c->out);
  if (c->part) cudaFree(c->part);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" fc2dgpu_ctx* fc2dgpu_ctx_create(int device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    fc3dgpu_set_error("fc2dgpu_ctx_create: no CUDA device %d", device);
    return nullptr;
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    fc3dgpu_set_error("fc2dgpu_ctx_create: cudaSetDevice(%d) failed", device);
    return nullptr;
  }
  fc2dgpu_ctx* c = new fc2dgpu_ctx();
  c->device = device;
  bool ok = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreate(&c->ev[0]) == cudaSuccess && cudaEventCreate(&c->ev[1]) == cudaSuccess &&
            cudaMalloc(&c->trace, sizeof(double) * TRACE_CAP) == cudaSuccess &&
            cudaMalloc(&c->out, sizeof(double) * 8) == cudaSuccess &&
            cudaMalloc(&c->part, sizeof(double) * 2 * GRID_MAX * 4) == cudaSuccess;
  if (!ok) {
    fc3dgpu_set_error("fc2dgpu_ctx_create: set-up failed (%s)", cudaGetErrorString(cudaGetLastError()));
    fc2dgpu_ctx_destroy(c);
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

extern "C" int fc2dgpu_ctx_set_problem(fc2dgpu_ctx* c, int nc, const int64_t* rowptr, const int64_t* colidx,
                                       const double* blocks, const double* q, const double* mu, int colour_kind) {
  if (!c || nc <= 0 || !rowptr || !colidx || !blocks || !q || !mu) {
    fc3dgpu_set_error("fc2dgpu_ctx_set_problem: invalid argument");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  const int64_t nnzb = rowptr[nc];
  if (rowptr[0] != 0 || nnzb < nc || nnzb > INT32_MAX) {
    fc3dgpu_set_error("fc2dgpu_ctx_set_problem: bad row pointer");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  std::vector<int> dposo(nc, -1);
  for (int i = 0; i < nc; i++) {
    if (rowptr[i + 1] < rowptr[i]) {
      fc3dgpu_set_error("fc2dgpu_ctx_set_problem: row pointer decreases at %d", i);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
      if (colidx[k] < 0 || colidx[k] >= nc) {
        fc3dgpu_set_error("fc2dgpu_ctx_set_problem: column index %lld out of range", (long long)colidx[k]);
        return NUMERICS_ERR_INVALID_ARGUMENT;
      }
      if (colidx[k] == i && dposo[i] < 0) dposo[i] = (int)(k - rowptr[i]);
    }
    if (dposo[i] < 0) {
      fc3dgpu_set_error("fc2dgpu_ctx_set_problem: contact %d has no diagonal block", i);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
  }
  for (int i = 0; i < nc; i++)
    if (!(mu[i] >= 0.0) || isinf(mu[i])) {
      fc3dgpu_set_error("fc2dgpu_ctx_set_problem: mu[%d] = %g is not a friction coefficient", i, mu[i]);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
  // colouring of the conflict graph (the device Jones-Plassmann colouring)
  std::vector<int32_t> colour(nc);
  const int ncol = fc3dgpu_colour(nc, rowptr, colidx, colour_kind, colour.data());
  if (ncol < 0) return ncol;
  if (ncol > MAXC) {
    fc3dgpu_set_error("fc2dgpu_ctx_set_problem: %d colours (at most %d)", ncol, MAXC);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (cudaSetDevice(c->device) != cudaSuccess) {
    fc3dgpu_set_error("fc2dgpu_ctx_set_problem: cudaSetDevice failed");
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
  std::vector<double> W((size_t)nnzb * 4), det(nc), qp(2 * (size_t)nc), mup(nc);
  bool singular = false;
  for (int p = 0; p < nc; p++) {
    const int i = c->perm[p];
    const int64_t k0 = rowptr[i], k1 = rowptr[i + 1];
    rp[p + 1] = rp[p] + (int)(k1 - k0);
    for (int64_t k = k0; k < k1; k++) {
      const int s = rp[p] + (int)(k - k0);
      col[s] = c->iperm[colidx[k]];
      for (int e = 0; e < 4; e++) W[4 * (size_t)s + e] = blocks[4 * k + e];
    }
    dpos[p] = dposo[i];
    const double* b = &blocks[4 * (rowptr[i] + dposo[i])];
    det[p] = b[0] * b[3] - b[1] * b[2];
    if (det[p] < DBL_EPSILON) singular = true;
    qp[2 * p] = q[2 * i];
    qp[2 * p + 1] = q[2 * i + 1];
    mup[p] = mu[i];
  }
  double s2 = 0.0;
  for (int64_t k = 0; k < 2LL * nc; k++) s2 += q[k] * q[k];
  c->norm_q = sqrt(s2);
  std::vector<double> zero(2 * (size_t)nc, 0.0);
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = upload(&c->cptr, cptr);
  if (e == cudaSuccess) e = upload(&c->rp, rp);
  if (e == cudaSuccess) e = upload(&c->col, col);
  if (e == cudaSuccess) e = upload(&c->dpos, dpos);
  if (e == cudaSuccess) e = upload(&c->W, W);
  if (e == cudaSuccess) e = upload(&c->det, det);
  if (e == cudaSuccess) e = upload(&c->q, qp);
  if (e == cudaSuccess) e = upload(&c->mu, mup);
  if (e == cudaSuccess) e = upload(&c->r, zero);
  if (e == cudaSuccess) e = upload(&c->u, zero);
  // FP32 copies; the determinants of the rounded blocks, in FP32
  {
    std::vector<float> W32(W.begin(), W.end()), det32(nc), q32(qp.begin(), qp.end()), mu32(mup.begin(), mup.end());
    for (int p = 0; p < nc; p++) {
      const float* b = &W32[4 * ((size_t)rp[p] + dpos[p])];
      det32[p] = b[0] * b[3] - b[1] * b[2];
    }
    std::vector<float> zero32(2 * (size_t)nc, 0.0f);
    if (e == cudaSuccess) e = upload(&c->W32, W32);
    if (e == cudaSuccess) e = upload(&c->det32, det32);
    if (e == cudaSuccess) e = upload(&c->q32, q32);
    if (e == cudaSuccess) e = upload(&c->mu32, mu32);
    if (e == cudaSuccess) e = upload(&c->r32, zero32);
  }
  if (e != cudaSuccess) {
    free_problem(c);
    fc3dgpu_set_error("fc2dgpu_ctx_set_problem: %s", cudaGetErrorString(e));
    return NUMERICS_ERR_UNKNOWN;
  }
  c->nc = nc;
  c->ncol = ncol;
  c->singular = singular;
  c->max_colour = 0;
  for (int k = 0; k < ncol; k++) c->max_colour = std::max(c->max_colour, cptr[k + 1] - cptr[k]);
  choose_shape(c);
  return 0;
}

extern "C" int fc2dgpu_ctx_set_q_mu(fc2dgpu_ctx* c, const double* q, const double* mu) {
  if (!c || !q || !mu || c->nc == 0) {
    fc3dgpu_set_error("fc2dgpu_ctx_set_q_mu: invalid argument");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  const int nc = c->nc;
  for (int i = 0; i < nc; i++)
    if (!(mu[i] >= 0.0) || isinf(mu[i])) {
      fc3dgpu_set_error("fc2dgpu_ctx_set_q_mu: mu[%d] = %g is not a friction coefficient", i, mu[i]);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
  std::vector<double> qp(2 * (size_t)nc), mup(nc);
  double s2 = 0.0;
  for (int64_t k = 0; k < 2LL * nc; k++) s2 += q[k] * q[k];
  for (int i = 0; i < nc; i++) {
    const size_t p = (size_t)c->iperm[i];
    qp[2 * p] = q[2 * i];
    qp[2 * p + 1] = q[2 * i + 1];
    mup[p] = mu[i];
  }
  K2(cudaSetDevice(c->device));
  K2(cudaMemcpy(c->q, qp.data(), sizeof(double) * qp.size(), cudaMemcpyHostToDevice));
  K2(cudaMemcpy(c->mu, mup.data(), sizeof(double) * mup.size(), cudaMemcpyHostToDevice));
  const std::vector<float> q32(qp.begin(), qp.end()), mu32(mup.begin(), mup.end());
  K2(cudaMemcpy(c->q32, q32.data(), sizeof(float) * q32.size(), cudaMemcpyHostToDevice));
  K2(cudaMemcpy(c->mu32, mu32.data(), sizeof(float) * mu32.size(), cudaMemcpyHostToDevice));
  c->norm_q = sqrt(s2);
  return 0;
}

extern "C" int fc2dgpu_ctx_set_r(fc2dgpu_ctx* c, const double* r) {
  if (!c || !r || c->nc == 0) return NUMERICS_ERR_INVALID_ARGUMENT;
  std::vector<double> rp(2 * (size_t)c->nc);
  for (int i = 0; i < c->nc; i++) {
    rp[2 * (size_t)c->iperm[i]] = r[2 * i];
    rp[2 * (size_t)c->iperm[i] + 1] = r[2 * i + 1];
  }
  K2(cudaSetDevice(c->device));
  K2(cudaMemcpy(c->r, rp.data(), sizeof(double) * rp.size(), cudaMemcpyHostToDevice));
  return 0;
}

// Launch shape: a cluster of up to CS_MAX blocks.  The sweep is bound by
// the latency of each colour's dependent chain (loads, FP64 divisions,
// barrier) and by the FP64 pipes (about two FP64 operations per clock per SM
// on this part), so a colour with more contacts is spread over more SMs;
// blocks of up to NT_MAX threads keep each thread on one or two contacts per
// colour.  The reactions are replicated in every block's shared memory when
// 16 bytes per contact fit (up to about 13,000 contacts), else kept in HBM.
static cudaLaunchConfig_t config(fc2dgpu_ctx* c, int cs, int nt, size_t smem, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(cs, 1, 1);
  cfg.blockDim = dim3(nt, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = c->stream;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

static size_t rep_bytes(const fc2dgpu_ctx* c) { return sizeof(double2) * (size_t)c->nc; }

// Kernel attributes a launch of this shape needs (cluster size above the
// portable 8, dynamic shared memory above 48 KiB).
template <typename K>
static cudaError_t prepare(K kernel, int cs, size_t smem) {
  cudaError_t e = cudaSuccess;
  if (cs > 8) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e == cudaSuccess && smem > 0) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return e;
}

// Whether a cluster of cs blocks of nt threads of the sweep kernel (the
// larger of the two kernels) can be resident on this device.
static bool cluster_fits(fc2dgpu_ctx* c, int cs, int nt, bool rep) {
  const size_t smem = rep ? rep_bytes(c) : 0;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = config(c, cs, nt, smem, attr);
  int n = 0;
  cudaError_t e = rep ? prepare(k_fc2d_nsgs<double, true, ClusterTeam>, cs, smem) : prepare(k_fc2d_nsgs<double, false, ClusterTeam>, cs, smem);
  if (e == cudaSuccess)
    e = rep ? cudaOccupancyMaxActiveClusters(&n, k_fc2d_nsgs<double, true, ClusterTeam>, &cfg)
            : cudaOccupancyMaxActiveClusters(&n, k_fc2d_nsgs<double, false, ClusterTeam>, &cfg);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return n > 0;
}

// A colour with more contacts than a full cluster has threads (16 x 512)
// goes to a cooperative grid over every SM instead (grid barrier, about
// 1-2 us, instead of the cluster's 0.3 us; the FP64 pipes of all SMs).
constexpr int GRID_FROM = CS_MAX * NT_MAX;

static void choose_grid(fc2dgpu_ctx* c) {
  int nt = c->nt_req > 0 ? c->nt_req : 256;
  nt = std::min(std::max(nt / 32 * 32, 32), NT_MAX);
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fc2d_nsgs<double, false, GridTeam>, nt, 0);
  const int resident = std::max(1, std::min(per_sm * sms, GRID_MAX));
  c->grid = true;
  c->rep = false;
  c->nt = nt;
  c->cs = 1;
  c->blocks = std::max(1, std::min((c->max_colour + nt - 1) / nt, resident));
}

static void choose_shape(fc2dgpu_ctx* c) {
  if (c->cs_req < 0 || (c->cs_req == 0 && c->rep_req != 2 && c->max_colour > GRID_FROM)) {
    choose_grid(c);
    return;
  }
  c->grid = false;
  int cs = c->cs_req, nt = c->nt_req;
  if (cs <= 0) {
    const int want = (c->max_colour + 63) / 64;  // about 64 contacts per SM and colour
    cs = 1;
    while (cs < want && cs < CS_MAX) cs *= 2;
  }
  cs = std::min(std::max(cs, 1), CS_MAX);
  if (nt <= 0) nt = std::min(NT_MAX, std::max(32, ((c->max_colour + cs - 1) / cs + 31) / 32 * 32));
  nt = std::min(std::max(nt / 32 * 32, 32), NT_MAX);
  // a replicated copy costs one distributed shared-memory store per block of
  // the cluster for each update: it pays for clusters of up to 4 blocks
  bool rep = c->rep_req == 2 || (c->rep_req == 0 && rep_bytes(c) <= REP_MAX_BYTES && cs <= 4);
  if (rep && c->rep_req == 0 && !cluster_fits(c, cs, nt, true)) rep = false;
  if (c->cs_req <= 0)
    while (cs > 1 && !cluster_fits(c, cs, nt, rep)) cs /= 2;
  c->cs = cs;
  c->nt = nt;
  c->rep = rep;
}

template <typename K, typename A>
static cudaError_t launch_grid(fc2dgpu_ctx* c, K kernel, const A& a) {
  void* params[] = {(void*)&a};
  return cudaLaunchCooperativeKernel((const void*)kernel, dim3(c->blocks), dim3(c->nt), params, 0, c->stream);
}

template <typename K, typename A>
static cudaError_t launch(fc2dgpu_ctx* c, K kernel, const A& a, size_t smem) {
  cudaError_t e = prepare(kernel, c->cs, smem);
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = config(c, c->cs, c->nt, smem, attr);
  return cudaLaunchKernelEx(&cfg, kernel, a);
}

extern "C" int fc2dgpu_ctx_set_launch(fc2dgpu_ctx* c, int cluster_blocks, int threads, int reactions) {
  if (!c || cluster_blocks < -1 || cluster_blocks > CS_MAX || threads < 0 || threads > NT_MAX ||
      (threads && threads % 32) || reactions < 0 || reactions > 2 || (cluster_blocks < 0 && reactions == 2)) {
    fc3dgpu_set_error("fc2dgpu_ctx_set_launch: cluster of 0..%d blocks (-1: cooperative grid, reactions in HBM), 0 or "
                      "32..%d threads (multiple of 32), reactions 0, 1 or 2", CS_MAX, NT_MAX);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (reactions == 2 && (c->nc == 0 || rep_bytes(c) > REP_MAX_BYTES)) {
    fc3dgpu_set_error("fc2dgpu_ctx_set_launch: %d contacts do not fit a shared-memory copy", c->nc);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (cluster_blocks > 0) {
    const bool rep = reactions == 2 || (reactions == 0 && c->nc > 0 && rep_bytes(c) <= REP_MAX_BYTES);
    if (cudaSetDevice(c->device) != cudaSuccess || !cluster_fits(c, cluster_blocks, threads ? threads : NT_MAX, rep)) {
      fc3dgpu_set_error("fc2dgpu_ctx_set_launch: a cluster of %d blocks of %d threads does not fit this device",
                        cluster_blocks, threads ? threads : NT_MAX);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
  }
  c->cs_req = cluster_blocks;
  c->nt_req = threads;
  c->rep_req = reactions;
  if (c->nc > 0) choose_shape(c);
  return 0;
}

extern "C" int fc2dgpu_ctx_launch_shape(fc2dgpu_ctx* c, int* cluster_blocks, int* threads, int* reactions) {
  if (!c) return NUMERICS_ERR_INVALID_ARGUMENT;
  if (cluster_blocks) *cluster_blocks = c->grid ? -c->blocks : c->cs;
  if (threads) *threads = c->nt;
  if (reactions) *reactions = c->rep ? 2 : 1;
  return 0;
}

static Args<double> args64(const fc2dgpu_ctx* c) {
  Args<double> a;
  memset(&a, 0, sizeof(a));
  a.nc = c->nc;
  a.ncol = c->ncol;
  a.cptr = c->cptr;
  a.rp = c->rp;
  a.col = c->col;
  a.dpos = c->dpos;
  a.W = c->W;
  a.det = c->det;
  a.q = c->q;
  a.mu = c->mu;
  a.r = c->r;
  a.rw = c->r;
  a.u = c->u;
  a.norm_q = c->norm_q;
  a.trace = c->trace;
  a.out = c->out;
  a.part = c->part;
  return a;
}

static Args<float> args32(const fc2dgpu_ctx* c) {
  Args<float> a;
  memset(&a, 0, sizeof(a));
  a.nc = c->nc;
  a.ncol = c->ncol;
  a.cptr = c->cptr;
  a.rp = c->rp;
  a.col = c->col;
  a.dpos = c->dpos;
  a.W = c->W32;
  a.det = c->det32;
  a.q = c->q32;
  a.mu = c->mu32;
  a.r = c->r;
  a.rw = c->r32;
  a.u = c->u;
  a.norm_q = c->norm_q;
  a.trace = c->trace;
  a.out = c->out + 4;
  a.part = c->part;
  return a;
}

extern "C" int fc2dgpu_ctx_set_precision(fc2dgpu_ctx* c, int precision, double switch_tol, int stall_window) {
  if (!c || precision < 0 || precision > 1 || !(switch_tol >= 0.0) || stall_window < 0) {
    fc3dgpu_set_error("fc2dgpu_ctx_set_precision: precision 0 or 1, switch_tol >= 0, stall_window >= 0");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  c->precision = precision;
  c->switch_tol = switch_tol;
  c->stall = stall_window > 0 ? stall_window : 64;
  return 0;
}

extern "C" int fc2dgpu_ctx_last_sweeps(fc2dgpu_ctx* c, int* sweeps32, int* sweeps64) {
  if (!c) return NUMERICS_ERR_INVALID_ARGUMENT;
  if (sweeps32) *sweeps32 = c->sweeps32;
  if (sweeps64) *sweeps64 = c->sweeps64;
  return 0;
}

extern "C" int fc2dgpu_ctx_compute_error(fc2dgpu_ctx* c, double norm_q, double* error) {
  if (!c || c->nc == 0 || !error) {
    fc3dgpu_set_error("fc2dgpu_ctx_compute_error: invalid argument");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  K2(cudaSetDevice(c->device));
  Args<double> a = args64(c);
  a.norm_q = norm_q;
  K2(c->grid ? launch_grid(c, k_fc2d_error<false, GridTeam>, a)
     : c->rep ? launch(c, k_fc2d_error<true, ClusterTeam>, a, rep_bytes(c))
              : launch(c, k_fc2d_error<false, ClusterTeam>, a, 0));
  K2(cudaMemcpyAsync(error, c->out + 1, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  K2(cudaStreamSynchronize(c->stream));
  return 0;
}

extern "C" int fc2dgpu_ctx_solve(fc2dgpu_ctx* c, double tol, int max_iter, int error_evaluation, int* iters,
                                 double* error, int* info, double* ms) {
  if (!c || c->nc == 0) {
    fc3dgpu_set_error("fc2dgpu_ctx_solve: no problem");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (max_iter < 0) {
    fc3dgpu_set_error("fc2dgpu_ctx_solve: negative iteration budget");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (c->singular) {
    // as fc2d_nsgs: a diagonal block with a determinant below DBL_EPSILON
    if (iters) *iters = 0;
    if (error) *error = INFINITY;
    if (info) *info = 1;
    if (ms) *ms = 0.0;
    c->trace_len = 0;
    return 0;
  }
  K2(cudaSetDevice(c->device));
  Args<double> a = args64(c);
  a.tol = tol;
  a.max_iter = max_iter;
  a.mode = error_evaluation == SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT_WITH_FULL_FINAL ? FULL_FINAL
           : error_evaluation == SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT                ? LIGHT
                                                                                               : NO_EVAL;
  // mixed precision: FP32 sweeps first (for the two modes that stop on an
  // error), then the FP64 sweeps of the reference's loop from their iterate,
  // on the budget and trace position the FP32 phase leaves (read on the
  // device: both launches go out back to back)
  const bool mixed = c->precision == 0 && a.mode != NO_EVAL && max_iter > 0;
  K2(cudaEventRecord(c->ev[0], c->stream));
  if (mixed) {
    Args<float> b = args32(c);
    b.tol = tol;
    b.max_iter = max_iter;
    b.mode = FP32_PHASE;
    b.switch_tol = c->switch_tol > 0.0 ? c->switch_tol : std::max(tol, 1e-6);
    b.stall = c->stall;
    K2(c->grid  ? launch_grid(c, k_fc2d_nsgs<float, false, GridTeam>, b)
       : c->rep ? launch(c, k_fc2d_nsgs<float, true, ClusterTeam>, b, sizeof(float2) * (size_t)c->nc)
                : launch(c, k_fc2d_nsgs<float, false, ClusterTeam>, b, 0));
    a.before = c->out + 4;
  }
  K2(c->grid  ? launch_grid(c, k_fc2d_nsgs<double, false, GridTeam>, a)
     : c->rep ? launch(c, k_fc2d_nsgs<double, true, ClusterTeam>, a, rep_bytes(c))
              : launch(c, k_fc2d_nsgs<double, false, ClusterTeam>, a, 0));
  K2(cudaEventRecord(c->ev[1], c->stream));
  double out[8];
  K2(cudaMemcpyAsync(out, c->out, sizeof(out), cudaMemcpyDeviceToHost, c->stream));
  K2(cudaStreamSynchronize(c->stream));
  float t = 0.f;
  cudaEventElapsedTime(&t, c->ev[0], c->ev[1]);
  if (iters) *iters = (int)out[0];
  if (error) *error = out[1];
  if (info) *info = (int)out[2];
  if (ms) *ms = t;
  c->sweeps32 = mixed ? (int)out[4] : 0;
  c->sweeps64 = (int)out[0] - c->sweeps32;
  c->trace_len = std::min((int)out[0], TRACE_CAP);
  return 0;
}

extern "C" int fc2dgpu_ctx_get_r_u(fc2dgpu_ctx* c, double* r, double* u) {
  if (!c || c->nc == 0) return NUMERICS_ERR_INVALID_ARGUMENT;
  K2(cudaSetDevice(c->device));
  std::vector<double> rp(2 * (size_t)c->nc), up(2 * (size_t)c->nc);
  K2(cudaMemcpy(rp.data(), c->r, sizeof(double) * rp.size(), cudaMemcpyDeviceToHost));
  K2(cudaMemcpy(up.data(), c->u, sizeof(double) * up.size(), cudaMemcpyDeviceToHost));
  for (int i = 0; i < c->nc; i++) {
    const size_t p = (size_t)c->iperm[i];
    if (r) {
      r[2 * i] = rp[2 * p];
      r[2 * i + 1] = rp[2 * p + 1];
    }
    if (u) {
      u[2 * i] = up[2 * p];
      u[2 * i + 1] = up[2 * p + 1];
    }
  }
  return 0;
}

extern "C" int fc2dgpu_ctx_colours(fc2dgpu_ctx* c, int32_t* colour) {
  if (!c || c->nc == 0) return NUMERICS_ERR_INVALID_ARGUMENT;
  if (colour) memcpy(colour, c->colour.data(), sizeof(int32_t) * c->nc);
  return c->ncol;
}

extern "C" int fc2dgpu_ctx_trace(fc2dgpu_ctx* c, double* out, int cap) {
  if (!c) return -1;
  const int n = std::min(cap, c->trace_len);
  if (n <= 0 || !out) return 0;
  K2(cudaSetDevice(c->device));
  K2(cudaMemcpy(out, c->trace, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return n;
}
