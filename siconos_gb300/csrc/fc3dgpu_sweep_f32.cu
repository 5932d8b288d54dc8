// float instantiations of the persistent coloured NSGS kernel.
#include "fc3dgpu_batch.cuh"
#include "fc3dgpu_flow.cuh"
#include "fc3dgpu_sweep.cuh"
#include "fc3dgpu_sweep_launch.h"

namespace fc3dgpu {
void warm_sweep_kernels_f64();

// The grid is queried at every launch (a few microseconds of host work
// against a solve of milliseconds): no launch state is kept between calls, so
// contexts on different host threads and devices never share any.
template <int T>
static cudaError_t launch_t(const SweepArgs<float>& a, int max_grid, size_t smem, cudaStream_t s, int* grid) {
  auto kern = nsgs_kernel<float, T>;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BlockDim<float>::value, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int g = nsm * per_sm;
  if (max_grid > 0 && g > max_grid) g = max_grid;
  if (g > 1024) g = 1024;
  *grid = g;
  void* args[] = {(void*)&a};
  return cudaLaunchCooperativeKernel((const void*)kern, dim3(g), dim3(BlockDim<float>::value), args, smem, s);
}

template <int T>
static int grid_t() {
  int dev = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nsgs_kernel<float, T>, BlockDim<float>::value, 0);
  return nsm * per_sm;
}

cudaError_t launch_sweep_f32(const SweepArgs<float>& a, int lanes, int max_grid, size_t smem, cudaStream_t s,
                             int* grid) {
  switch (lanes) {
    case 1: return launch_t<1>(a, max_grid, smem, s, grid);
    case 2: return launch_t<2>(a, max_grid, 0, s, grid);
    case 4: return launch_t<4>(a, max_grid, 0, s, grid);
    case 8: return launch_t<8>(a, max_grid, 0, s, grid);
    default: return cudaErrorInvalidValue;
  }
}

void warm_sweep_kernels() {
  cudaFuncAttributes fa;
  cudaFuncGetAttributes(&fa, nsgs_kernel<float, 1>);
  cudaFuncGetAttributes(&fa, nsgs_kernel<float, 2>);
  cudaFuncGetAttributes(&fa, nsgs_kernel<float, 4>);
  cudaFuncGetAttributes(&fa, nsgs_kernel<float, 8>);
  cudaFuncGetAttributes(&fa, nsgs_flow_kernel<12>);
  cudaFuncGetAttributes(&fa, nsgs_flow_kernel<10>);
  cudaFuncGetAttributes(&fa, nsgs_flow_kernel<8>);
  warm_sweep_kernels_f64();
}

int sweep_grid_f32(int lanes) {
  switch (lanes) {
    case 1: return grid_t<1>();
    case 2: return grid_t<2>();
    case 4: return grid_t<4>();
    case 8: return grid_t<8>();
    default: return 0;
  }
}

// Warps per block of the dataflow sweep that fit the shared memory of an SM
// with per-warp buffers for slabs of up to maxslot slots: the largest of
// `want` (8, 10 or 12; 0 = 10, the default) and the smaller counts that fit,
// else 0.  On the 60x60x30 lattice 10 warps were measured the fastest with
// round-trip polls of the slab counters; the autotuner measures 8, 10 and 12.
int flow_warps(int maxslot, int want) {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t room = optin > 4096 ? (size_t)optin - 4096 : 0;  // static shared memory of the kernel
  const size_t buf = flow_buf_bytes(maxslot);
  if (want <= 0) want = 10;
  const int cand[3] = {12, 10, 8};
  for (int nw : cand)
    if (nw <= want && (size_t)nw * buf <= room) return nw;
  return 0;
}

template <int NW>
static cudaError_t launch_flow_t(const SweepArgs<float>& a, const FlowArgs& f, cudaStream_t s, int* grid) {
  auto kern = nsgs_flow_kernel<NW>;
  const size_t smem = (size_t)NW * f.buf_bytes;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NW * 32, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int g = nsm;  // one block per SM: each holds NW per-warp buffers
  if (g > 1024) g = 1024;
  *grid = g;
  void* args[] = {(void*)&a, (void*)&f};
  return cudaLaunchCooperativeKernel((const void*)kern, dim3(g), dim3(NW * 32), args, smem, s);
}

cudaError_t launch_flow_f32(const SweepArgs<float>& a, const FlowArgs& f, int nw, cudaStream_t s, int* grid) {
  switch (nw) {
    case 12: return launch_flow_t<12>(a, f, s, grid);
    case 10: return launch_flow_t<10>(a, f, s, grid);
    case 8: return launch_flow_t<8>(a, f, s, grid);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t pack_flow_records(int nslab, const long long* slab_off, const int* slab_nslot, const float* W,
                              const int* col, const float* q, const float* D, const float* mu, const float* rho,
                              const long long* rec_off, float* rec, cudaStream_t s) {
  if (nslab <= 0) return cudaSuccess;
  const int grid = nslab < 4096 ? nslab : 4096;
  k_flow_pack<<<grid, 256, 0, s>>>(nslab, slab_off, slab_nslot, W, col, q, D, mu, rho, rec_off, rec);
  return cudaGetLastError();
}

cudaError_t build_flow_deps(int nslab, int npad, int ncol, const int* sptr_d, const int* perm, const int* slab_nslot,
                            const long long* slab_off, const int* col, const int* dptr, int* count, int* dep,
                            cudaStream_t s) {
  k_flow_deps<<<(nslab + 127) / 128, 128, 0, s>>>(nslab, npad, ncol, sptr_d, perm, slab_nslot, slab_off, col, dptr,
                                                  count, dep);
  return cudaGetLastError();
}

// Resident blocks of the batched kernel on the current device, queried
// outside any stream capture; the caller keeps the figure with its context.
cudaError_t batch_grid_f32(int* grid) {
  auto kern = nsgs_batch_kernel<float>;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BlockDim<float>::value, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  *grid = nsm * per_sm;
  return cudaSuccess;
}

// One block per problem, at most max_grid (batch_grid_f32) resident blocks.
cudaError_t launch_batch_f32(const BatchArgs<float>& b, int max_grid, cudaStream_t s, int* grid) {
  if (max_grid < 1) return cudaErrorInvalidConfiguration;
  const int g = max_grid < b.nscenes ? max_grid : b.nscenes;
  *grid = g;
  nsgs_batch_kernel<float><<<g, BlockDim<float>::value, 0, s>>>(b);
  return cudaGetLastError();
}

void warm_batch_kernel_f32() {
  cudaFuncAttributes fa;
  cudaFuncGetAttributes(&fa, nsgs_batch_kernel<float>);
}

}  // namespace fc3dgpu
