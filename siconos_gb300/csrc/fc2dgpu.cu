// Coloured NSGS for 2D friction contact on the GPU (include/fc2dgpu.h).
//
// Layout: contacts permuted by colour (stable in contact order); per permuted
// row its blocks in the caller's order (diagonal included, at dpos), each a
// 2x2 column-major block, with the permuted column index; q, mu, r, u in
// permuted order.  One thread block per problem: within a colour each
// thread takes contacts p = lo + tid, lo + tid + blockDim, ...; a block
// barrier separates colours.  FP64 without FMA contraction, in the
// reference's operation order.
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

constexpr int NT = 512;
constexpr int MAXC = 128;
constexpr int TRACE_CAP = 1 << 16;

struct Args {
  int nc, ncol;
  const int* cptr;    // ncol + 1 permuted-row bounds of the colours
  const int* rp;      // nc + 1 slot pointer per permuted row
  const int* col;     // permuted column of each slot
  const int* dpos;    // offset in the row of its first diagonal block
  const double* W;    // 4 per slot
  const double* det;  // determinant of each row's diagonal block
  const double* q;
  const double* mu;
  double* r;
  double* u;
  double norm_q, tol;
  int max_iter;
  int mode;  // 0 light with full final, 1 light, 2 no evaluation
  double* trace;
  double* out;  // [0] sweeps, [1] final error, [2] info, [3] last light error
};

__device__ __forceinline__ void mvp2x2(const double* a, const double* v, double* y) {
  y[0] += a[0] * v[0];
  y[1] += a[1] * v[0];
  y[0] += a[2] * v[1];
  y[1] += a[3] * v[1];
}

// Fixed-order block sum of n values per thread (xor-shuffle tree in each
// warp, then the warps in order): the same for a given block shape.
template <int N>
__device__ __forceinline__ void block_sum(double v[N]) {
  __shared__ double sh[NT / 32][N];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < N; i++) {
    double x = v[i];
    for (int o = 16; o >= 1; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sh[w][i] = x;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < N; i++) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k][i];
    v[i] = s;
  }
  __syncthreads();
}

// fc2d_compute_error (fc2d_compute_error.c:40-140): u = q + W r block by
// block (per block w_i = 1.0 w_i + 1.0 (a_i0 r0 + a_i1 r1), the reference's
// 2x2 gemv), natural-map error, relative to max(|r|, |u|, |q|).
__device__ double full_error(const Args& a) {
  double v[3] = {0.0, 0.0, 0.0};
  for (int p = threadIdx.x; p < a.nc; p += blockDim.x) {
    double w[2] = {a.q[2 * p], a.q[2 * p + 1]};
    for (int s = a.rp[p]; s < a.rp[p + 1]; s++) {
      const double* blk = a.W + 4 * (size_t)s;
      const double* x = a.r + 2 * (size_t)a.col[s];
      for (int i = 0; i < 2; i++) {
        double t = 0.0;
        t += blk[i] * x[0];
        t += blk[2 + i] * x[1];
        w[i] = 1.0 * w[i] + 1.0 * t;
      }
    }
    a.u[2 * p] = w[0];
    a.u[2 * p + 1] = w[1];
    const double r0 = a.r[2 * p], r1 = a.r[2 * p + 1], mu = a.mu[p];
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
  block_sum<3>(v);
  double e = sqrt(v[0]);
  const double scal = fmax(sqrt(v[1]), fmax(sqrt(v[2]), a.norm_q));
  if (fabs(scal) > DBL_EPSILON) e /= scal;
  return e;
}

// fc2d_nsgs_local_solve (fc2d_nsgs.c:212-252)
__device__ __forceinline__ void local_solve(const double* W, double D, const double* q, double mu, double* P) {
  const double Wnn = W[0], Wtn = W[1], Wnt = W[2], Wtt = W[3];
  if (q[0] > 0) {
    P[0] = 0;
    P[1] = 0;
  } else {
    P[0] = -(Wtt * q[0] - Wnt * q[1]) / D;
    P[1] = -(-Wtn * q[0] + Wnn * q[1]) / D;
    const double muPn = mu * P[0];
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

__global__ void __launch_bounds__(NT, 1) k_fc2d_nsgs(const Args a) {
  double tolerance = a.tol, err = INFINITY;
  int iter = 0, not_conv = 1;
  while (iter < a.max_iter && not_conv) {
    ++iter;
    double v[2] = {0.0, 0.0};
    for (int c = 0; c < a.ncol; c++) {
      for (int p = a.cptr[c] + threadIdx.x; p < a.cptr[c + 1]; p += blockDim.x) {
        const double old0 = a.r[2 * p], old1 = a.r[2 * p + 1];
        double ql[2] = {a.q[2 * p], a.q[2 * p + 1]};
        const int s0 = a.rp[p], s1 = a.rp[p + 1], sd = s0 + a.dpos[p];
        // every block on the diagonal is left out (SBM_row_prod_no_diag_2x2)
        for (int s = s0; s < s1; s++) {
          const int j = a.col[s];
          if (j != p) mvp2x2(a.W + 4 * (size_t)s, a.r + 2 * (size_t)j, ql);
        }
        double P[2] = {old0, old1};
        local_solve(a.W + 4 * (size_t)sd, a.det[p], ql, a.mu[p], P);
        const double x0 = old0 - P[0], x1 = old1 - P[1];
        v[0] += x0 * x0 + x1 * x1;
        a.r[2 * p] = P[0];
        a.r[2 * p + 1] = P[1];
      }
      __syncthreads();
    }
    for (int p = threadIdx.x; p < a.nc; p += blockDim.x) v[1] += a.r[2 * p] * a.r[2 * p] + a.r[2 * p + 1] * a.r[2 * p + 1];
    block_sum<2>(v);
    err = sqrt(v[0]);
    const double nr = sqrt(v[1]);
    if (fabs(nr) > DBL_EPSILON) err /= nr;
    if (a.trace && threadIdx.x == 0 && iter <= TRACE_CAP) a.trace[iter - 1] = err;
    if (a.mode == 1) {
      not_conv = !(err < tolerance);  // determine_convergence (fc2d_nsgs.c:147-162)
    } else if (a.mode == 0 && err < tolerance) {
      // determine_convergence_with_full_final (fc2d_nsgs.c:187-228)
      not_conv = 0;
      const double full = full_error(a);
      if (full > a.tol) {
        tolerance = err / full * a.tol;
        not_conv = 1;
      }
    }
  }
  const double light = err;
  if (a.mode == 0) {
    err = full_error(a);
    not_conv = !(err < a.tol);
  } else if (a.mode == 2) {
    err = INFINITY;  // no branch of the sweep loop evaluates an error (fc2d_nsgs.c:438-448)
    not_conv = 1;
  }
  if (threadIdx.x == 0) {
    a.out[0] = iter;
    a.out[1] = err;
    a.out[2] = not_conv;
    a.out[3] = light;
  }
}

__global__ void __launch_bounds__(NT, 1) k_fc2d_error(const Args a) {
  const double e = full_error(a);
  if (threadIdx.x == 0) a.out[1] = e;
}

}  // namespace fc2dgpu

// ---------------------------------------------------------------------------
// Context (C-ABI)
// ---------------------------------------------------------------------------
using namespace fc2dgpu;

struct fc2dgpu_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  int nc = 0, ncol = 0;
  bool singular = false;
  double norm_q = 0.0;
  std::vector<int> perm, iperm, colour;
  int *cptr = nullptr, *rp = nullptr, *col = nullptr, *dpos = nullptr;
  double *W = nullptr, *det = nullptr, *q = nullptr, *mu = nullptr, *r = nullptr, *u = nullptr, *trace = nullptr,
         *out = nullptr;
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

static void free_problem(fc2dgpu_ctx* c) {
  void* ptrs[] = {c->cptr, c->rp, c->col, c->dpos, c->W, c->det, c->q, c->mu, c->r, c->u};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  c->cptr = c->rp = c->col = c->dpos = nullptr;
  c->W = c->det = c->q = c->mu = c->r = c->u = nullptr;
  c->nc = 0;
}

extern "C" void fc2dgpu_ctx_destroy(fc2dgpu_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  free_problem(c);
  if (c->trace) cudaFree(c->trace);
  if (c->out) cudaFree(c->out);
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
            cudaMalloc(&c->out, sizeof(double) * 8) == cudaSuccess;
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
  if (e != cudaSuccess) {
    free_problem(c);
    fc3dgpu_set_error("fc2dgpu_ctx_set_problem: %s", cudaGetErrorString(e));
    return NUMERICS_ERR_UNKNOWN;
  }
  c->nc = nc;
  c->ncol = ncol;
  c->singular = singular;
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

static Args args_of(const fc2dgpu_ctx* c) {
  Args a;
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
  a.u = c->u;
  a.norm_q = c->norm_q;
  a.trace = c->trace;
  a.out = c->out;
  return a;
}

extern "C" int fc2dgpu_ctx_compute_error(fc2dgpu_ctx* c, double norm_q, double* error) {
  if (!c || c->nc == 0 || !error) {
    fc3dgpu_set_error("fc2dgpu_ctx_compute_error: invalid argument");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  K2(cudaSetDevice(c->device));
  Args a = args_of(c);
  a.norm_q = norm_q;
  k_fc2d_error<<<1, NT, 0, c->stream>>>(a);
  K2(cudaGetLastError());
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
  Args a = args_of(c);
  a.tol = tol;
  a.max_iter = max_iter;
  a.mode = error_evaluation == SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT_WITH_FULL_FINAL ? 0
           : error_evaluation == SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT                ? 1
                                                                                               : 2;
  K2(cudaEventRecord(c->ev[0], c->stream));
  k_fc2d_nsgs<<<1, NT, 0, c->stream>>>(a);
  K2(cudaGetLastError());
  K2(cudaEventRecord(c->ev[1], c->stream));
  double out[4];
  K2(cudaMemcpyAsync(out, c->out, sizeof(out), cudaMemcpyDeviceToHost, c->stream));
  K2(cudaStreamSynchronize(c->stream));
  float t = 0.f;
  cudaEventElapsedTime(&t, c->ev[0], c->ev[1]);
  if (iters) *iters = (int)out[0];
  if (error) *error = out[1];
  if (info) *info = (int)out[2];
  if (ms) *ms = t;
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
