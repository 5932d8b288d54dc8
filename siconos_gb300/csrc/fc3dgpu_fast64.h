// Launchers of the FP64 sweep kernels built with the fast one-contact
// arithmetic (fc3dgpu_sweep_f64fast.cu, the opt-in fast FP64 polish).  The
// kernels there are the kernels of fc3dgpu_sweep_f64.cu compiled in their own
// namespace with FC3D_FAST_F64: the argument structs they take are the same
// definitions (fc3dgpu_layout.cuh, fc3dgpu_batch_args.cuh), passed here by
// address so the two namespaces' types never meet in one translation unit.
#pragma once
#include <cuda_runtime.h>

// args: a fc3dgpu::SweepArgs<double>; lanes 1, 2, 4 or 8; as launch_sweep_f64.
cudaError_t fc3dgpu_launch_sweep_f64_fast(const void* args, int lanes, int max_grid, cudaStream_t s, int* grid);
// args: a fc3dgpu::BatchArgs<double>; as launch_batch_f64 / batch_grid_f64.
cudaError_t fc3dgpu_launch_batch_f64_fast(const void* args, int max_grid, cudaStream_t s, int* grid);
cudaError_t fc3dgpu_batch_grid_f64_fast(int* grid);
