// Launchers of the persistent sweep kernel, one translation unit per
// precision: the FP64 unit is compiled with --fmad=false so its arithmetic
// is the CPU restatement's, the FP32 unit keeps FMA contraction.
#pragma once
#include <cuda_runtime.h>

#include "fc3dgpu_layout.cuh"

namespace fc3dgpu {
// Cooperative launch with as many resident blocks as fit (capped by
// max_grid when > 0).  Returns the cudaError_t of the launch; *grid gets the
// number of blocks.
// smem: dynamic shared memory of the launch (staging buffers), 0 when off
cudaError_t launch_sweep_f32(const SweepArgs<float>& a, int lanes, int max_grid, size_t smem, cudaStream_t s,
                             int* grid);
cudaError_t launch_sweep_f64(const SweepArgs<double>& a, int lanes, int max_grid, size_t smem, cudaStream_t s,
                             int* grid);
int sweep_grid_f32(int lanes);
void warm_sweep_kernels();
template <typename Real>
struct BatchArgs;
// Batched kernel: resident blocks on the current device (query outside any
// stream capture), and the launch of min(max_grid, problems) blocks.
cudaError_t batch_grid_f32(int* grid);
cudaError_t batch_grid_f64(int* grid);
cudaError_t launch_batch_f32(const BatchArgs<float>& b, int max_grid, cudaStream_t s, int* grid);
cudaError_t launch_batch_f64(const BatchArgs<double>& b, int max_grid, cudaStream_t s, int* grid);
void warm_batch_kernel_f32();
void warm_batch_kernel_f64();
int sweep_grid_f64(int lanes);
// Slab-dataflow FP32 sweep: warps per block for slabs of up to maxslot
// slots, at most `want` (0: the default; 0 returned: the per-warp buffers do
// not fit), its cooperative launch (one block per SM), and the build of its
// per-slab column lists (k_flow_deps).
int flow_warps(int maxslot, int want);
cudaError_t launch_flow_f32(const SweepArgs<float>& a, const FlowArgs& f, int nw, cudaStream_t s, int* grid);
// The dataflow sweep's per-slab records from the layout's FP32 arrays.
cudaError_t pack_flow_records(int nslab, const long long* slab_off, const int* slab_nslot, const float* W,
                              const int* col, const float* q, const float* D, const float* mu, const float* rho,
                              const long long* rec_off, float* rec, cudaStream_t s);
cudaError_t build_flow_deps(int nslab, int npad, int ncol, const int* sptr_d, const int* perm, const int* slab_nslot,
                            const long long* slab_off, const int* col, const int* dptr, int* count, int* dep,
                            cudaStream_t s);
}  // namespace fc3dgpu
