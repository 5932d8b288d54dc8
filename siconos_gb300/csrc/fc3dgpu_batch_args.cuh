// BatchArgs for host code (the batched kernel itself is in fc3dgpu_batch.cuh).
#pragma once
#include "fc3dgpu_layout.cuh"

namespace fc3dgpu {

template <typename Real>
struct BatchArgs {
  SweepArgs<Real> base;      // layout, state, controls (sptr/ncol unused)
  int nscenes;
  const int* order;          // problems by decreasing size
  const int* scene_ncol;
  const int* scene_sptr;     // nscenes x (FC3D_MAX_COLOURS + 1), absolute slab indices
  const double* scene_normq; // |q| of each problem
  const int* scene_budget;   // sweep budget of each problem (nullptr: base.max_sweeps)
  int* queue;                // next problem index, zero at launch
  double* scene_out;         // nscenes x 8: sweeps, incr, full error, info, working tol, local tol
  // outputs of the previous (FP32) phase, or nullptr: a problem whose FP32
  // iterate met the tolerance gets its FP64 error checked before any sweep
  const double* scene_out_prev;
};

}  // namespace fc3dgpu
