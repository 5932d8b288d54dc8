// double instantiations of the persistent coloured NSGS kernel.
#include "fc3dgpu_batch.cuh"
#include "fc3dgpu_sweep.cuh"
#include "fc3dgpu_sweep_launch.h"

namespace fc3dgpu {

// The grid is queried at every launch (a few microseconds of host work
// against a solve of milliseconds): no launch state is kept between calls, so
// contexts on different host threads and devices never share any.
template <int T>
static cudaError_t launch_t(const SweepArgs<double>& a, int max_grid, size_t smem, cudaStream_t s, int* grid) {
  auto kern = nsgs_kernel<double, T>;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BlockDim<double>::value, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int g = nsm * per_sm;
  if (max_grid > 0 && g > max_grid) g = max_grid;
  if (g > 1024) g = 1024;
  *grid = g;
  void* args[] = {(void*)&a};
  return cudaLaunchCooperativeKernel((const void*)kern, dim3(g), dim3(BlockDim<double>::value), args, smem, s);
}

template <int T>
static int grid_t() {
  int dev = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nsgs_kernel<double, T>, BlockDim<double>::value, 0);
  return nsm * per_sm;
}

cudaError_t launch_sweep_f64(const SweepArgs<double>& a, int lanes, int max_grid, size_t smem, cudaStream_t s,
                             int* grid) {
  switch (lanes) {
    case 1: return launch_t<1>(a, max_grid, smem, s, grid);
    case 2: return launch_t<2>(a, max_grid, 0, s, grid);
    case 4: return launch_t<4>(a, max_grid, 0, s, grid);
    case 8: return launch_t<8>(a, max_grid, 0, s, grid);
    default: return cudaErrorInvalidValue;
  }
}

void warm_sweep_kernels_f64() {
  cudaFuncAttributes fa;
  cudaFuncGetAttributes(&fa, nsgs_kernel<double, 1>);
  cudaFuncGetAttributes(&fa, nsgs_kernel<double, 2>);
  cudaFuncGetAttributes(&fa, nsgs_kernel<double, 4>);
  cudaFuncGetAttributes(&fa, nsgs_kernel<double, 8>);
}

int sweep_grid_f64(int lanes) {
  switch (lanes) {
    case 1: return grid_t<1>();
    case 2: return grid_t<2>();
    case 4: return grid_t<4>();
    case 8: return grid_t<8>();
    default: return 0;
  }
}

// Resident blocks of the batched kernel on the current device, queried
// outside any stream capture; the caller keeps the figure with its context.
cudaError_t batch_grid_f64(int* grid) {
  auto kern = nsgs_batch_kernel<double>;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BlockDim<double>::value, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  *grid = nsm * per_sm;
  return cudaSuccess;
}

// One block per problem, at most max_grid (batch_grid_f64) resident blocks.
cudaError_t launch_batch_f64(const BatchArgs<double>& b, int max_grid, cudaStream_t s, int* grid) {
  if (max_grid < 1) return cudaErrorInvalidConfiguration;
  const int g = max_grid < b.nscenes ? max_grid : b.nscenes;
  *grid = g;
  nsgs_batch_kernel<double><<<g, BlockDim<double>::value, 0, s>>>(b);
  return cudaGetLastError();
}

void warm_batch_kernel_f64() {
  cudaFuncAttributes fa;
  cudaFuncGetAttributes(&fa, nsgs_batch_kernel<double>);
}

}  // namespace fc3dgpu
