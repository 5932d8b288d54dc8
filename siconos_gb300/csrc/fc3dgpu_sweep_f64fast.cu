// FP64 sweep kernels with the fast one-contact arithmetic: the persistent
// coloured kernel and the batched kernel of fc3dgpu_sweep_f64.cu, compiled
// with FC3D_FAST_F64 so the local solver's FP64 divisions and square roots
// come from FP32 seeds refined by one Newton-Raphson step in FP64
// (fc3dgpu_local.cuh) instead of the exactly rounded operations.  The
// natural-map error, the light error and the tolerance logic are unchanged,
// so convergence is still decided on the FP64 fc3d_compute_error.  The
// kernels are put in their own namespace (the token fc3dgpu is renamed for
// the included headers) so they do not clash with the exact ones.
#define FC3D_FAST_F64 1
#define fc3dgpu fc3dgpu_fast64
#include "fc3dgpu_batch.cuh"
#include "fc3dgpu_sweep.cuh"
#undef fc3dgpu

#include "fc3dgpu_fast64.h"

namespace fc3dgpu_fast64 {

template <int T>
static cudaError_t launch_t(const SweepArgs<double>& a, int max_grid, cudaStream_t s, int* grid) {
  auto kern = nsgs_kernel<double, T>;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BlockDim<double>::value, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int g = nsm * per_sm;
  if (max_grid > 0 && g > max_grid) g = max_grid;
  if (g > 1024) g = 1024;
  *grid = g;
  void* args[] = {(void*)&a};
  return cudaLaunchCooperativeKernel((const void*)kern, dim3(g), dim3(BlockDim<double>::value), args, 0, s);
}

}  // namespace fc3dgpu_fast64

cudaError_t fc3dgpu_launch_sweep_f64_fast(const void* args, int lanes, int max_grid, cudaStream_t s, int* grid) {
  using namespace fc3dgpu_fast64;
  const SweepArgs<double>& a = *static_cast<const SweepArgs<double>*>(args);
  switch (lanes) {
    case 1: return launch_t<1>(a, max_grid, s, grid);
    case 2: return launch_t<2>(a, max_grid, s, grid);
    case 4: return launch_t<4>(a, max_grid, s, grid);
    case 8: return launch_t<8>(a, max_grid, s, grid);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t fc3dgpu_batch_grid_f64_fast(int* grid) {
  using namespace fc3dgpu_fast64;
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

cudaError_t fc3dgpu_launch_batch_f64_fast(const void* args, int max_grid, cudaStream_t s, int* grid) {
  using namespace fc3dgpu_fast64;
  const BatchArgs<double>& b = *static_cast<const BatchArgs<double>*>(args);
  if (max_grid < 1) return cudaErrorInvalidConfiguration;
  const int g = max_grid < b.nscenes ? max_grid : b.nscenes;
  *grid = g;
  nsgs_batch_kernel<double><<<g, BlockDim<double>::value, 0, s>>>(b);
  return cudaGetLastError();
}
