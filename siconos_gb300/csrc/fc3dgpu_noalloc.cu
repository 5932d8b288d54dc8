// fc3d_compute_error on a problem that is already in device memory, with no
// device allocation at all: the variant of the solver's error evaluation
// (u = q + W r and the natural-map residual, reduced over all contacts)
// whose scratch -- per-chunk partial sums and a completion ticket -- lives in
// a fixed file-scope device array instead of buffers owned by a context.
//
// Callers that cannot let a library allocate: applications that hand all
// device memory to their own pool (a cudaMalloc or cudaFree would synchronise
// the device and stall their other streams in the middle of a time step, or
// fail because the pool has taken the memory).
//
// The reduction order is fixed by the chunking (256 contacts per chunk,
// chunks summed in index order), so the result does not depend on the grid.
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include <mutex>

#include "fc3dgpu.h"
#include "fc3dgpu_local.cuh"

extern "C" void fc3dgpu_set_error(const char* fmt, ...);

namespace fc3dgpu {
namespace noalloc {

constexpr int CHUNK = 256;  // contacts per chunk = threads per block
constexpr int MAX_CHUNKS = FC3DGPU_NOALLOC_MAX_CONTACTS / CHUNK;
static_assert(MAX_CHUNKS * CHUNK == FC3DGPU_NOALLOC_MAX_CONTACTS, "limit must be a multiple of the chunk");
// 3 partial sums per chunk, then one 256-byte line holding the ticket
constexpr int SCRATCH_DOUBLES = 3 * MAX_CHUNKS + 32;
static_assert(SCRATCH_DOUBLES * 8 == FC3DGPU_NOALLOC_SCRATCH_BYTES, "header states the scratch size");

static __device__ __align__(256) double g_scratch[SCRATCH_DOUBLES];

__device__ __forceinline__ void block_sum3(double v[3], double (*sh)[3]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sh[w][k] = x;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 3; k++) {
    double s = 0.0;
    for (int i = 0; i < CHUNK / 32; i++) s += sh[i][k];
    v[k] = s;
  }
  __syncthreads();
}

// Rows are read in the caller's block-CSR order (the diagonal block at its
// own position), as SBM_gemv_3x3 does (SparseBlockMatrix.c:360-419).  A row
// pointer or column index out of range is not followed: the error becomes
// NaN.
__global__ void __launch_bounds__(CHUNK) k_error_noalloc(int nc, long long nnz, const int64_t* __restrict__ rowptr,
                                                         const int64_t* __restrict__ colidx,
                                                         const double* __restrict__ blocks,
                                                         const double* __restrict__ q, const double* __restrict__ mu,
                                                         const double* __restrict__ r, double norm_q,
                                                         double* __restrict__ velocity, double* __restrict__ error,
                                                         double* __restrict__ scratch) {
  __shared__ double sh[CHUNK / 32][3];
  __shared__ int last;
  __shared__ int bad_any;
  double* part = scratch;
  unsigned* ticket = reinterpret_cast<unsigned*>(scratch + 3 * MAX_CHUNKS);
  unsigned* bad = ticket + 1;
  const int nchunks = (nc + CHUNK - 1) / CHUNK;
  int badl = 0;
  for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const int i = ch * CHUNK + threadIdx.x;
    double v[3] = {0.0, 0.0, 0.0};
    if (i < nc) {
      double u[3] = {q[3 * (size_t)i], q[3 * (size_t)i + 1], q[3 * (size_t)i + 2]};
      const double rr[3] = {r[3 * (size_t)i], r[3 * (size_t)i + 1], r[3 * (size_t)i + 2]};
      const long long b0 = rowptr[i], b1 = rowptr[i + 1];
      if (b0 < 0 || b1 < b0 || b1 > nnz) {
        badl = 1;
      } else {
        for (long long b = b0; b < b1; b++) {
          const long long j = colidx[b];
          if (j < 0 || j >= nc) {
            badl = 1;
            continue;
          }
          double wv[9];
#pragma unroll
          for (int e = 0; e < 9; e++) wv[e] = blocks[9 * b + e];
          const double rj[3] = {r[3 * j], r[3 * j + 1], r[3 * j + 2]};
          mvp3x3(wv, rj, u);
        }
      }
      v[0] = unitary_error2(rr, u, mu[i]);
      v[1] = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
      v[2] = rr[0] * rr[0] + rr[1] * rr[1] + rr[2] * rr[2];
      if (velocity) {
        velocity[3 * (size_t)i] = u[0];
        velocity[3 * (size_t)i + 1] = u[1];
        velocity[3 * (size_t)i + 2] = u[2];
      }
    }
    block_sum3(v, sh);
    if (threadIdx.x == 0) {
      part[3 * ch] = v[0];
      part[3 * ch + 1] = v[1];
      part[3 * ch + 2] = v[2];
    }
  }
  if (__syncthreads_or(badl) && threadIdx.x == 0) atomicOr(bad, 1u);
  // the last block to finish sums the chunk partials in chunk order
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double v[3] = {0.0, 0.0, 0.0};
  for (int ch = threadIdx.x; ch < nchunks; ch += CHUNK) {
    v[0] += __ldcg(&part[3 * ch]);
    v[1] += __ldcg(&part[3 * ch + 1]);
    v[2] += __ldcg(&part[3 * ch + 2]);
  }
  block_sum3(v, sh);
  if (threadIdx.x == 0) bad_any = (int)atomicOr(bad, 0u);
  __syncthreads();
  if (threadIdx.x == 0) {
    double e = sqrt(v[0]);
    const double scal = fmax(norm_q, fmax(sqrt(v[2]), sqrt(v[1])));
    if (fabs(scal) > DBL_EPSILON) e /= scal;
    *error = bad_any ? __longlong_as_double(0x7ff8000000000000LL) : e;
    // leave the ticket and the flag at zero for the next call
    *ticket = 0u;
    *bad = 0u;
  }
}

// Address of g_scratch and SM count per device, looked up at the first call
// with that device current.  The address belongs to the CUDA context that was
// current then (the device's primary context, unless the caller made another
// driver context current): the entry is keyed by that context and looked up
// again when another context is current, e.g. after cudaDeviceReset.
constexpr int MAX_DEVICES = 64;
std::mutex g_mutex;
struct Entry {
  void* ctx;
  double* addr;
  int sms;
};
Entry g_entry[MAX_DEVICES];
typedef int (*CtxGetCurrent)(void**);  // cuCtxGetCurrent, through the runtime
CtxGetCurrent g_ctx_current = nullptr;

static void* current_context() {
  void* ctx = nullptr;
  if (g_ctx_current && g_ctx_current(&ctx) != 0) ctx = nullptr;
  return ctx;
}

int setup(int dev, double** addr, int* sms) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_ctx_current) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      cudaGetLastError();
      fc3dgpu_set_error("fc3dgpu_compute_error_device: cuCtxGetCurrent is not available");
      return NUMERICS_ERR_NOT_IMPLEMENTED;
    }
    g_ctx_current = reinterpret_cast<CtxGetCurrent>(fn);
  }
  Entry& en = g_entry[dev];
  void* ctx = current_context();
  if (!en.addr || !ctx || ctx != en.ctx) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      fc3dgpu_set_error("fc3dgpu_compute_error_device: cudaGetSymbolAddress on device %d: %s", dev,
                        cudaGetErrorString(e));
      return NUMERICS_ERR_UNKNOWN;
    }
    int n = 0;
    e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess || n <= 0) {
      cudaGetLastError();
      fc3dgpu_set_error("fc3dgpu_compute_error_device: SM count of device %d: %s", dev, cudaGetErrorString(e));
      return NUMERICS_ERR_UNKNOWN;
    }
    en.ctx = current_context();  // the look-up made the primary context current if none was
    en.sms = n;
    en.addr = static_cast<double*>(p);
  }
  *addr = en.addr;
  *sms = en.sms;
  return 0;
}

// Memory a kernel on device dev may read or write through p as given: device
// memory of that device (memory of another device is refused, since peer
// access may be off), managed memory, or mapped pinned host memory whose
// device address is p itself.
bool device_accessible(const void* p, int dev) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  switch (at.type) {
    case cudaMemoryTypeDevice: return at.device == dev;
    case cudaMemoryTypeManaged: return true;
    case cudaMemoryTypeHost: return at.devicePointer == p;
    default: return false;
  }
}

}  // namespace noalloc
}  // namespace fc3dgpu

extern "C" int fc3dgpu_compute_error_device(int nc, int64_t nnz, const int64_t* rowptr, const int64_t* colidx,
                                            const double* blocks, const double* q, const double* mu,
                                            const double* reaction, double norm_q, double* velocity, double* error,
                                            void* stream) {
  using namespace fc3dgpu::noalloc;
  if (nc < 0 || nnz < 0) {
    fc3dgpu_set_error("fc3dgpu_compute_error_device: negative size (nc = %d, nnz = %lld)", nc, (long long)nnz);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (nc > FC3DGPU_NOALLOC_MAX_CONTACTS) {
    fc3dgpu_set_error(
        "fc3dgpu_compute_error_device: %d contacts exceed the limit of %d (FC3DGPU_NOALLOC_MAX_CONTACTS); use "
        "fc3dgpu_ctx_compute_error",
        nc, FC3DGPU_NOALLOC_MAX_CONTACTS);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (!error || !rowptr || (nc > 0 && (!q || !mu || !reaction)) || (nnz > 0 && (!colidx || !blocks))) {
    fc3dgpu_set_error("fc3dgpu_compute_error_device: null pointer");
    return NUMERICS_ERR_NULL_POINTER;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    fc3dgpu_set_error("fc3dgpu_compute_error_device: no current CUDA device (%s)", cudaGetErrorString(e));
    return NUMERICS_ERR_NOT_IMPLEMENTED;
  }
  if (dev < 0 || dev >= MAX_DEVICES) {
    fc3dgpu_set_error("fc3dgpu_compute_error_device: device %d beyond %d", dev, MAX_DEVICES);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  const void* ptrs[] = {rowptr, colidx, blocks, q, mu, reaction, velocity, error};
  for (const void* p : ptrs)
    if (p && !device_accessible(p, dev)) {
      fc3dgpu_set_error("fc3dgpu_compute_error_device: %p is not memory device %d can access", p, dev);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
  double* scratch = nullptr;
  int sms = 0;
  int rc = setup(dev, &scratch, &sms);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the ticket and the bad-input flag must be zero at launch; a launch that
  // completes leaves them zero, this makes an interrupted one harmless
  e = cudaMemsetAsync(scratch + 3 * MAX_CHUNKS, 0, 2 * sizeof(unsigned), s);
  if (e == cudaSuccess) {
    const int nchunks = (nc + CHUNK - 1) / CHUNK;
    int grid = 4 * sms;
    if (grid > nchunks) grid = nchunks;
    if (grid < 1) grid = 1;
    k_error_noalloc<<<grid, CHUNK, 0, s>>>(nc, (long long)nnz, rowptr, colidx, blocks, q, mu, reaction, norm_q,
                                           velocity, error, scratch);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    fc3dgpu_set_error("fc3dgpu_compute_error_device: %s", cudaGetErrorString(e));
    return NUMERICS_ERR_UNKNOWN;
  }
  return 0;
}
