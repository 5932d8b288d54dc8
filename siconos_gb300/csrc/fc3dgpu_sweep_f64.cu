// double instantiations of the persistent coloured NSGS kernel.
#include "fc3dgpu_batch.cuh"
#include "fc3dgpu_sweep.cuh"
#include "fc3dgpu_sweep_launch.h"

namespace fc3dgpu {

template <int T>
static cudaError_t launch_t(const SweepArgs<double>& a, int max_grid, size_t smem, cudaStream_t s, int* grid) {
  auto kern = nsgs_kernel<double, T>;
  static int cached_dev = -1, cached_g = 0;
  static size_t cached_smem = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (cached_dev != dev || cached_smem != smem) {
    int nsm = 0, per_sm = 0;
    e = cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BlockDim<double>::value, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    cached_g = nsm * per_sm;
    cached_dev = dev;
    cached_smem = smem;
  }
  int g = cached_g;
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

static int batch_cached_dev_f64 = -1, batch_cached_g_f64 = 0;

// Occupancy of the batched kernel, queried outside any stream capture.
cudaError_t prepare_batch_f64() {
  auto kern = nsgs_batch_kernel<double>;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (batch_cached_dev_f64 == dev) return cudaSuccess;
  e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BlockDim<double>::value, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  batch_cached_g_f64 = nsm * per_sm;
  batch_cached_dev_f64 = dev;
  return cudaSuccess;
}

cudaError_t launch_batch_f64(const BatchArgs<double>& b, cudaStream_t s, int* grid) {
  auto kern = nsgs_batch_kernel<double>;
  int& cached_dev = batch_cached_dev_f64;
  int& cached_g = batch_cached_g_f64;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (cached_dev != dev) {
    int nsm = 0, per_sm = 0;
    e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BlockDim<double>::value, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    cached_g = nsm * per_sm;
    cached_dev = dev;
  }
  int g = cached_g < b.nscenes ? cached_g : b.nscenes;
  *grid = g;
  kern<<<g, BlockDim<double>::value, 0, s>>>(b);
  return cudaGetLastError();
}

void warm_batch_kernel_f64() {
  cudaFuncAttributes fa;
  cudaFuncGetAttributes(&fa, nsgs_batch_kernel<double>);
}

}  // namespace fc3dgpu
