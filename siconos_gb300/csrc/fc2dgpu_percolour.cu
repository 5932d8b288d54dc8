// The reference's per-colour GPU design for 2D friction contact (see
// include/fc2dgpu_percolour.h): cuSPARSE SpMV + local-solve kernel per
// colour, one CUDA graph per sweep, convergence tested on the host.
#include <cuda_runtime.h>
#include <cusparse.h>
#include <float.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <numeric>
#include <vector>

#include "fc2dgpu_percolour.h"
#include "fc3dgpu.h"

extern "C" void fc3dgpu_set_error(const char* fmt, ...);

namespace {

constexpr int TPB = 256;

__global__ void k_local_solve_colour(const double* __restrict__ Wd, const double* __restrict__ det,
                                     const double* __restrict__ y, const double* __restrict__ qc,
                                     const double* __restrict__ mu, double* __restrict__ z, double* sumP2,
                                     double* sumErr2, int k1, int k2) {
  __shared__ double sh[2][TPB];
  const int i = k1 + blockIdx.x * blockDim.x + threadIdx.x;
  double p2 = 0.0, e2 = 0.0;
  if (i < k2) {
    const double q0 = y[2 * i] + qc[2 * i], q1 = y[2 * i + 1] + qc[2 * i + 1];
    const double* w = Wd + 4 * (size_t)i;
    const double Wnn = w[0], Wtn = w[1], Wnt = w[2], Wtt = w[3], D = det[i], m = mu[i];
    const double o0 = z[2 * i], o1 = z[2 * i + 1];
    double P0, P1;
    if (q0 > 0.0) {
      P0 = 0.0;
      P1 = 0.0;
    } else {
      P0 = -(Wtt * q0 - Wnt * q1) / D;
      P1 = -(-Wtn * q0 + Wnn * q1) / D;
      const double muPn = m * P0;
      if (fabs(P1) > muPn) {
        if (P1 + muPn < 0.0) {
          P0 = -q0 / (Wnn - m * Wnt);
          P1 = -m * P0;
        } else {
          P0 = -q0 / (Wnn + m * Wnt);
          P1 = m * P0;
        }
      }
    }
    z[2 * i] = P0;
    z[2 * i + 1] = P1;
    p2 = P0 * P0 + P1 * P1;
    e2 = (P0 - o0) * (P0 - o0) + (P1 - o1) * (P1 - o1);
  }
  sh[0][threadIdx.x] = p2;
  sh[1][threadIdx.x] = e2;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + s];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicAdd(sumP2, sh[0][0]);
    atomicAdd(sumErr2, sh[1][0]);
  }
}

}  // namespace

struct fc2dgpu_percolour {
  int device = 0, nc = 0, ncol = 0;
  std::vector<int> perm, iperm, cptr;
  // the problem in contact order, for the host full error
  std::vector<int64_t> rowptr, colidx;
  std::vector<double> blocks, q, mu, z, u;
  double norm_q = 0.0;
  cudaStream_t stream = nullptr;
  cusparseHandle_t sp = nullptr;
  std::vector<cusparseSpMatDescr_t> mats;
  std::vector<cusparseDnVecDescr_t> ys;
  cusparseDnVecDescr_t zvec = nullptr;
  std::vector<void*> bufs;
  int64_t *d_ci = nullptr;
  double *d_val = nullptr, *d_Wd = nullptr, *d_det = nullptr, *d_q = nullptr, *d_mu = nullptr, *d_z = nullptr,
         *d_y = nullptr, *d_sum = nullptr;
  std::vector<void*> work;  // SpMV work buffers per colour (owned by bufs)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // the local-solve kernel loaded from a CUDA library image, when set
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kref = nullptr;
  // block-sparse sweep (the reference's BLOCKLEGACY variant): per colour a
  // BSR matvec of 2x2 blocks (diagonal blocks kept with zero values), int32
  // indices, launched each sweep without a graph
  bool bsr = false;
  cusparseMatDescr_t descr = nullptr;
  std::vector<int> bsr_cnnz;  // first block of each colour, and the end
  int *d_brp = nullptr, *d_bci = nullptr;
  double* d_bval = nullptr;
};

#define KP(x)                                                                             \
  do {                                                                                    \
    cudaError_t e_ = (x);                                                                 \
    if (e_ != cudaSuccess) {                                                              \
      fc3dgpu_set_error("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
      return NUMERICS_ERR_UNKNOWN;                                                        \
    }                                                                                     \
  } while (0)
#define SP(x)                                                                                \
  do {                                                                                       \
    cusparseStatus_t s_ = (x);                                                               \
    if (s_ != CUSPARSE_STATUS_SUCCESS) {                                                     \
      fc3dgpu_set_error("%s:%d %s: cuSPARSE status %d", __FILE__, __LINE__, #x, (int)s_); \
      return NUMERICS_ERR_UNKNOWN;                                                           \
    }                                                                                        \
  } while (0)

extern "C" void fc2dgpu_percolour_destroy(fc2dgpu_percolour* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  for (auto m : h->mats)
    if (m) cusparseDestroySpMat(m);
  for (auto y : h->ys)
    if (y) cusparseDestroyDnVec(y);
  if (h->zvec) cusparseDestroyDnVec(h->zvec);
  for (void* b : h->bufs)
    if (b) cudaFree(b);
  void* ptrs[] = {h->d_ci, h->d_val, h->d_Wd, h->d_det, h->d_q, h->d_mu, h->d_z, h->d_y, h->d_sum};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h->sp) cusparseDestroy(h->sp);
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->lib) cudaLibraryUnload(h->lib);
  if (h->descr) cusparseDestroyMatDescr(h->descr);
  void* bptrs[] = {h->d_brp, h->d_bci, h->d_bval};
  for (void* p : bptrs)
    if (p) cudaFree(p);
  delete h;
}

template <typename T>
static cudaError_t put(T** d, const std::vector<T>& v) {
  cudaError_t e = cudaMalloc((void**)d, sizeof(T) * std::max<size_t>(v.size(), 1));
  if (e == cudaSuccess && !v.empty()) e = cudaMemcpy(*d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
  return e;
}

// The local-solve kernel of colour range [lo, hi): this file's, or the loaded
// one with the same arguments.
static cudaError_t launch_local(fc2dgpu_percolour* h, int lo, int hi) {
  const int blocks = (hi - lo + TPB - 1) / TPB;
  if (h->kref) {
    const double *Wd = h->d_Wd, *det = h->d_det, *y = h->d_y, *qc = h->d_q, *mu = h->d_mu;
    double *z = h->d_z, *s0 = h->d_sum, *s1 = h->d_sum + 1;
    void* args[] = {&Wd, &det, &y, &qc, &mu, &z, &s0, &s1, &lo, &hi};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(TPB);
    cfg.dynamicSmemBytes = 2 * TPB * sizeof(double);
    cfg.stream = h->stream;
    return cudaLaunchKernelExC(&cfg, (const void*)h->kref, args);
  }
  k_local_solve_colour<<<blocks, TPB, 0, h->stream>>>(h->d_Wd, h->d_det, h->d_y, h->d_q, h->d_mu, h->d_z, h->d_sum,
                                                      h->d_sum + 1, lo, hi);
  return cudaGetLastError();
}

// One sweep as a CUDA graph: a memset of the two sums, then per colour the
// SpMV of its rows and the local-solve kernel (this file's, or the loaded
// one with the same arguments: 256 threads, 2 x 256 doubles of dynamic
// shared memory as fc2d_nsgs_graph_permut_cuda.cu:574-587 launches it).
static int capture(fc2dgpu_percolour* h) {
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  h->exec = nullptr;
  h->graph = nullptr;
  const double one = 1.0, zero = 0.0;
  KP(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  cudaMemsetAsync(h->d_sum, 0, sizeof(double) * 2, h->stream);
  cudaError_t le = cudaSuccess;
  for (int c = 0; c < h->ncol; c++) {
    if (!h->mats[c]) continue;
    cusparseSpMV(h->sp, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, h->mats[c], h->zvec, &zero, h->ys[c], CUDA_R_64F,
                 CUSPARSE_SPMV_ALG_DEFAULT, h->work[c]);
    const cudaError_t e = launch_local(h, h->cptr[c], h->cptr[c + 1]);
    if (le == cudaSuccess) le = e;
  }
  const cudaError_t ec = cudaStreamEndCapture(h->stream, &h->graph);
  KP(le);
  KP(ec);
  KP(cudaGraphInstantiate(&h->exec, h->graph, 0));
  return 0;
}

static int setup(fc2dgpu_percolour* h, int colour_kind) {
  const int nc = h->nc;
  std::vector<int32_t> colour(nc);
  const int ncol = fc3dgpu_colour(nc, h->rowptr.data(), h->colidx.data(), colour_kind, colour.data());
  if (ncol < 0) return ncol;
  h->ncol = ncol;
  h->perm.resize(nc);
  std::iota(h->perm.begin(), h->perm.end(), 0);
  std::stable_sort(h->perm.begin(), h->perm.end(), [&](int a, int b) { return colour[a] < colour[b]; });
  h->iperm.resize(nc);
  for (int p = 0; p < nc; p++) h->iperm[h->perm[p]] = p;
  h->cptr.assign(ncol + 1, 0);
  for (int i = 0; i < nc; i++) h->cptr[colour[i] + 1]++;
  for (int k = 0; k < ncol; k++) h->cptr[k + 1] += h->cptr[k];
  // permuted scalar CSR without the diagonal blocks (rows 2p, 2p + 1 for
  // permuted contact p), columns in the permuted numbering, sorted
  std::vector<int64_t> rp(2 * (size_t)nc + 1, 0), ci;
  std::vector<double> val, Wd(4 * (size_t)nc), det(nc), qp(2 * (size_t)nc), mup(nc);
  std::vector<std::pair<int, int64_t>> row;  // (permuted column block, source block)
  for (int p = 0; p < nc; p++) {
    const int i = h->perm[p];
    row.clear();
    int64_t dblk = -1;
    for (int64_t k = h->rowptr[i]; k < h->rowptr[i + 1]; k++) {
      if (h->colidx[k] == i) {
        if (dblk < 0) dblk = k;
        continue;
      }
      row.push_back({h->iperm[h->colidx[k]], k});
    }
    if (dblk < 0) {
      fc3dgpu_set_error("fc2dgpu_percolour_create: contact %d has no diagonal block", i);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
    std::sort(row.begin(), row.end());
    for (int a = 0; a < 2; a++) {
      for (auto& e : row)
        for (int b = 0; b < 2; b++) {
          ci.push_back(2 * (int64_t)e.first + b);
          val.push_back(h->blocks[4 * e.second + 2 * b + a]);
        }
      rp[2 * (size_t)p + a + 1] = (int64_t)ci.size();
    }
    for (int e = 0; e < 4; e++) Wd[4 * (size_t)p + e] = h->blocks[4 * dblk + e];
    const double* d = &h->blocks[4 * dblk];
    det[p] = d[0] * d[3] - d[1] * d[2];
    if (det[p] < DBL_EPSILON) {
      fc3dgpu_set_error("fc2dgpu_percolour_create: singular diagonal block at contact %d", i);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
    qp[2 * (size_t)p] = h->q[2 * (size_t)i];
    qp[2 * (size_t)p + 1] = h->q[2 * (size_t)i + 1];
    mup[p] = h->mu[i];
  }
  KP(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  KP(put(&h->d_ci, ci));
  KP(put(&h->d_val, val));
  KP(put(&h->d_Wd, Wd));
  KP(put(&h->d_det, det));
  KP(put(&h->d_q, qp));
  KP(put(&h->d_mu, mup));
  KP(cudaMalloc(&h->d_z, sizeof(double) * 2 * nc));
  KP(cudaMalloc(&h->d_y, sizeof(double) * 2 * nc));
  KP(cudaMalloc(&h->d_sum, sizeof(double) * 2));
  KP(cudaMemset(h->d_z, 0, sizeof(double) * 2 * nc));
  SP(cusparseCreate(&h->sp));
  SP(cusparseSetStream(h->sp, h->stream));
  SP(cusparseCreateDnVec(&h->zvec, 2 * (int64_t)nc, h->d_z, CUDA_R_64F));
  const double one = 1.0, zero = 0.0;
  h->mats.assign(ncol, nullptr);
  h->ys.assign(ncol, nullptr);
  std::vector<void*>& work = h->work;
  work.assign(ncol, nullptr);
  for (int c = 0; c < ncol; c++) {
    const int lo = h->cptr[c], n = h->cptr[c + 1] - lo;
    if (n == 0) continue;
    // the colour's rows, with a row pointer of their own
    const int64_t first = rp[2 * (size_t)lo], last = rp[2 * (size_t)(lo + n)];
    std::vector<int64_t> rpc(2 * (size_t)n + 1);
    for (size_t k = 0; k <= 2 * (size_t)n; k++) rpc[k] = rp[2 * (size_t)lo + k] - first;
    int64_t* d_rpc = nullptr;
    KP(put(&d_rpc, rpc));
    h->bufs.push_back(d_rpc);
    SP(cusparseCreateCsr(&h->mats[c], 2 * (int64_t)n, 2 * (int64_t)nc, last - first, d_rpc, h->d_ci + first,
                         h->d_val + first, CUSPARSE_INDEX_64I, CUSPARSE_INDEX_64I, CUSPARSE_INDEX_BASE_ZERO,
                         CUDA_R_64F));
    // the colour's products land at its own rows of y (global row index)
    SP(cusparseCreateDnVec(&h->ys[c], 2 * (int64_t)n, h->d_y + 2 * (size_t)lo, CUDA_R_64F));
    size_t sz = 0;
    SP(cusparseSpMV_bufferSize(h->sp, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, h->mats[c], h->zvec, &zero, h->ys[c],
                               CUDA_R_64F, CUSPARSE_SPMV_ALG_DEFAULT, &sz));
    KP(cudaMalloc(&work[c], std::max<size_t>(sz, 16)));
    h->bufs.push_back(work[c]);
  }
  return capture(h);
}

extern "C" fc2dgpu_percolour* fc2dgpu_percolour_create(int device, int nc, const int64_t* rowptr,
                                                       const int64_t* colidx, const double* blocks, const double* q,
                                                       const double* mu, int colour_kind) {
  if (nc <= 0 || !rowptr || !colidx || !blocks || !q || !mu || rowptr[0] != 0) {
    fc3dgpu_set_error("fc2dgpu_percolour_create: invalid argument");
    return nullptr;
  }
  for (int i = 0; i < nc; i++) {
    if (rowptr[i + 1] < rowptr[i]) {
      fc3dgpu_set_error("fc2dgpu_percolour_create: row pointer decreases");
      return nullptr;
    }
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++)
      if (colidx[k] < 0 || colidx[k] >= nc) {
        fc3dgpu_set_error("fc2dgpu_percolour_create: column index out of range");
        return nullptr;
      }
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    fc3dgpu_set_error("fc2dgpu_percolour_create: no CUDA device %d", device);
    return nullptr;
  }
  fc2dgpu_percolour* h = new fc2dgpu_percolour();
  h->device = device;
  h->nc = nc;
  const int64_t nnzb = rowptr[nc];
  h->rowptr.assign(rowptr, rowptr + nc + 1);
  h->colidx.assign(colidx, colidx + nnzb);
  h->blocks.assign(blocks, blocks + 4 * nnzb);
  h->q.assign(q, q + 2 * (size_t)nc);
  h->mu.assign(mu, mu + nc);
  h->z.assign(2 * (size_t)nc, 0.0);
  h->u.assign(2 * (size_t)nc, 0.0);
  double s2 = 0.0;
  for (double x : h->q) s2 += x * x;
  h->norm_q = sqrt(s2);
  if (setup(h, colour_kind) != 0) {
    fc2dgpu_percolour_destroy(h);
    return nullptr;
  }
  return h;
}

// fc2d_compute_error on the host, the reaction in contact order (the
// reference copies z back and evaluates it on the CPU).
static double host_full_error(fc2dgpu_percolour* h) {
  const int nc = h->nc;
  const double* z = h->z.data();
  double* w = h->u.data();
  for (size_t k = 0; k < 2 * (size_t)nc; k++) w[k] = h->q[k];
  for (int i = 0; i < nc; i++)
    for (int64_t k = h->rowptr[i]; k < h->rowptr[i + 1]; k++) {
      const double* a = &h->blocks[4 * k];
      const double* x = &z[2 * h->colidx[k]];
      for (int r = 0; r < 2; r++) {
        double s = 0.0;
        s += a[r] * x[0];
        s += a[2 + r] * x[1];
        w[2 * i + r] = 1.0 * w[2 * i + r] + 1.0 * s;
      }
    }
  double err = 0.0, nz = 0.0, nw = 0.0;
  for (int i = 0; i < nc; i++) {
    const double r0 = z[2 * i], r1 = z[2 * i + 1], u0 = w[2 * i], u1 = w[2 * i + 1], m = h->mu[i];
    double t0 = r0 - u0 - m * fabs(u1), t1 = r1 - u1;
    const double nT = fabs(t1);
    if (m * nT <= -t0) {
      t0 = 0.;
      t1 = 0.;
    } else if (nT > m * t0) {
      t0 = (m * nT + t0) / (m * m + 1.0);
      t1 = m * t0 * (double)((t1 > 0) - (t1 < 0));
    }
    t0 = r0 - t0;
    t1 = r1 - t1;
    err += t0 * t0 + t1 * t1;
  }
  for (size_t k = 0; k < 2 * (size_t)nc; k++) nz += z[k] * z[k];
  for (size_t k = 0; k < 2 * (size_t)nc; k++) nw += w[k] * w[k];
  err = sqrt(err);
  const double scal = fmax(sqrt(nz), fmax(sqrt(nw), h->norm_q));
  if (fabs(scal) > DBL_EPSILON) err /= scal;
  return err;
}

static int pull_z(fc2dgpu_percolour* h) {
  std::vector<double> zp(2 * (size_t)h->nc);
  KP(cudaMemcpy(zp.data(), h->d_z, sizeof(double) * zp.size(), cudaMemcpyDeviceToHost));
  for (int i = 0; i < h->nc; i++) {
    h->z[2 * (size_t)i] = zp[2 * (size_t)h->iperm[i]];
    h->z[2 * (size_t)i + 1] = zp[2 * (size_t)h->iperm[i] + 1];
  }
  return 0;
}

// One sweep of the block-sparse variant (fc2d_nsgs_graph_permut_cuda_blocklegacy.cu:533-567):
// the sums cleared, then per colour cusparseDbsrmv of its block rows (column-
// major 2x2 blocks) into y at its rows, and the local-solve kernel.
static int bsr_sweep(fc2dgpu_percolour* h) {
  const double one = 1.0, zero = 0.0;
  KP(cudaMemsetAsync(h->d_sum, 0, sizeof(double) * 2, h->stream));
  for (int c = 0; c < h->ncol; c++) {
    const int lo = h->cptr[c], hi = h->cptr[c + 1];
    if (hi == lo) continue;
    const int first = h->bsr_cnnz[c], nnz = h->bsr_cnnz[c + 1] - first;
    SP(cusparseDbsrmv(h->sp, CUSPARSE_DIRECTION_COLUMN, CUSPARSE_OPERATION_NON_TRANSPOSE, hi - lo, h->nc, nnz, &one,
                      h->descr, h->d_bval + 4 * (size_t)first, h->d_brp + lo + c, h->d_bci + first, 2, h->d_z, &zero,
                      h->d_y + 2 * (size_t)lo));
    KP(launch_local(h, lo, hi));
  }
  return 0;
}

extern "C" int fc2dgpu_percolour_use_bsr(fc2dgpu_percolour* h, int on) {
  if (!h) return NUMERICS_ERR_INVALID_ARGUMENT;
  KP(cudaSetDevice(h->device));
  if (on && !h->d_brp) {
    const int nc = h->nc;
    // permuted block rows in colour order, columns in the permuted numbering
    // (sorted), the diagonal block kept with zero values; per colour a row
    // pointer of its own (nc + colours entries)
    std::vector<int> rp, ci;
    std::vector<double> val;
    std::vector<std::pair<int, int64_t>> row;
    h->bsr_cnnz.assign(h->ncol + 1, 0);
    for (int c = 0; c < h->ncol; c++) {
      const int base = (int)ci.size();
      h->bsr_cnnz[c] = base;
      for (int p = h->cptr[c]; p < h->cptr[c + 1]; p++) {
        rp.push_back((int)ci.size() - base);
        const int i = h->perm[p];
        row.clear();
        for (int64_t k = h->rowptr[i]; k < h->rowptr[i + 1]; k++) row.push_back({h->iperm[h->colidx[k]], k});
        std::sort(row.begin(), row.end());
        for (auto& e : row) {
          ci.push_back(e.first);
          for (int t = 0; t < 4; t++) val.push_back(e.first == p ? 0.0 : h->blocks[4 * e.second + t]);
        }
      }
      rp.push_back((int)ci.size() - base);
    }
    h->bsr_cnnz[h->ncol] = (int)ci.size();
    KP(put(&h->d_brp, rp));
    KP(put(&h->d_bci, ci));
    KP(put(&h->d_bval, val));
    SP(cusparseCreateMatDescr(&h->descr));
    SP(cusparseSetMatIndexBase(h->descr, CUSPARSE_INDEX_BASE_ZERO));
    SP(cusparseSetMatType(h->descr, CUSPARSE_MATRIX_TYPE_GENERAL));
  }
  h->bsr = on != 0;
  return 0;
}

extern "C" int fc2dgpu_percolour_solve(fc2dgpu_percolour* h, const double* r0, double tol, int max_iter, int* iters,
                                       double* error, int* info, double* ms) {
  if (!h || max_iter < 0) return NUMERICS_ERR_INVALID_ARGUMENT;
  KP(cudaSetDevice(h->device));
  std::vector<double> zp(2 * (size_t)h->nc, 0.0);
  if (r0)
    for (int i = 0; i < h->nc; i++) {
      zp[2 * (size_t)h->iperm[i]] = r0[2 * i];
      zp[2 * (size_t)h->iperm[i] + 1] = r0[2 * i + 1];
    }
  KP(cudaMemcpy(h->d_z, zp.data(), sizeof(double) * zp.size(), cudaMemcpyHostToDevice));
  const auto t0 = std::chrono::steady_clock::now();
  double tolerance = tol, err = INFINITY;
  int iter = 0, not_conv = 1;
  while (iter < max_iter && not_conv) {
    if (h->bsr) {
      if (int rc = bsr_sweep(h)) return rc;
    } else {
      KP(cudaGraphLaunch(h->exec, h->stream));
    }
    double e2 = 0.0, p2 = 0.0;
    KP(cudaMemcpyAsync(&e2, h->d_sum + 1, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    KP(cudaStreamSynchronize(h->stream));
    KP(cudaMemcpyAsync(&p2, h->d_sum, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    KP(cudaStreamSynchronize(h->stream));
    err = sqrt(e2);
    const double nr = sqrt(p2);
    if (fabs(nr) > DBL_EPSILON) err /= nr;
    if (err < tolerance) {
      not_conv = 0;
      if (pull_z(h)) return NUMERICS_ERR_UNKNOWN;
      const double full = host_full_error(h);
      if (full > tol) {
        tolerance = err / full * tol;
        not_conv = 1;
      }
    }
    ++iter;
  }
  if (pull_z(h)) return NUMERICS_ERR_UNKNOWN;
  err = host_full_error(h);
  const auto t1 = std::chrono::steady_clock::now();
  if (iters) *iters = iter;
  if (error) *error = err;
  if (info) *info = err < tol ? 0 : 1;
  if (ms) *ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  return 0;
}

// The reference kernels' C++ names (five const double*, three double*, two
// const int): fc2d_nsgs_graph_permut_cuda.cu:213-223 and
// fc2d_nsgs_graph_permut_cuda_blocklegacy.cu:215-224.
static const char* const REF_KERNELS[] = {
    "_Z41fc2d_nsgs_local_solve_kernel_range_reducePKdS0_S0_S0_S0_PdS1_S1_ii",
    "_Z43fc2d_nsgs_local_solve_kernel_range_reduce_2PKdS0_S0_S0_S0_PdS1_S1_ii"};

extern "C" int fc2dgpu_percolour_use_kernel_file(fc2dgpu_percolour* h, const char* path) {
  if (!h || !path) return NUMERICS_ERR_INVALID_ARGUMENT;
  KP(cudaSetDevice(h->device));
  cudaLibrary_t lib = nullptr;
  cudaKernel_t k = nullptr;
  cudaError_t e = cudaLibraryLoadFromFile(&lib, path, nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();  // the failed load is reported here, not by a later launch check
    fc3dgpu_set_error("fc2dgpu_percolour_use_kernel_file: cannot load %s: %s", path, cudaGetErrorString(e));
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  for (const char* name : REF_KERNELS) {
    e = cudaLibraryGetKernel(&k, lib, name);
    if (e == cudaSuccess) break;
  }
  if (e != cudaSuccess) {
    cudaLibraryUnload(lib);
    cudaGetLastError();
    fc3dgpu_set_error("fc2dgpu_percolour_use_kernel_file: no reference local-solve kernel in %s", path);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  // the new sweep graph first: the old one (destroyed by capture) may
  // launch the old library's kernel
  cudaLibrary_t old = h->lib;
  h->lib = lib;
  h->kref = k;
  const int rc = capture(h);
  if (old) cudaLibraryUnload(old);
  return rc;
}

extern "C" int fc2dgpu_percolour_get_r_u(fc2dgpu_percolour* h, double* r, double* u) {
  if (!h) return NUMERICS_ERR_INVALID_ARGUMENT;
  if (r) memcpy(r, h->z.data(), sizeof(double) * h->z.size());
  if (u) memcpy(u, h->u.data(), sizeof(double) * h->u.size());
  return 0;
}
