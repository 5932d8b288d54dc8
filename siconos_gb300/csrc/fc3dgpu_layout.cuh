// Device layout of a coloured friction-contact problem, shared by the
// layout-building code and the sweep kernels.
//
// W of the reference is a SparseBlockStructuredMatrix: per block row, a list
// of scattered 3x3 column-major blocks (SparseBlockMatrix.h:82-121).  On the
// device the rows are permuted so that each colour is a contiguous range,
// padded to whole slabs of 32 rows, and each slab is stored slot-major
// (ELL within the slab):
//
//   W[(slab_off[s] + slot) * 9 + e][lane]   element e of the slot-th
//                                           off-diagonal block of row
//                                           32*s + lane (coalesced: one
//                                           128/256-byte line per (slot, e))
//   col[(slab_off[s] + slot)][lane]         permuted column of that block
//   D[(s * 9 + e)][lane], q[(s*3 + a)][lane], mu[s][lane], rho[(s*2+b)][lane]
//
// Padding rows (perm = -1) and padding slots (rows shorter than the slab's
// longest) hold zero blocks whose column is the extra zero entry of r at
// index npad, so the product needs no branch.
#pragma once
#include <stdint.h>

#define FC3D_SLAB 32
#define FC3D_MAX_COLOURS 128

namespace fc3dgpu {

template <typename Real>
struct SweepArgs {
  // layout
  int ncol;
  int nslab;
  int npad;                     // 32 * nslab
  int sptr[FC3D_MAX_COLOURS + 1];  // slab range of each colour
  int ccount[FC3D_MAX_COLOURS];    // contacts of each colour (rows past it in the range are padding)
  const int* slab_nslot;
  const long long* slab_off;
  const int* perm;              // padded permuted row -> original contact, -1 pad
  const int* dpos;              // slot position of the diagonal in the CSR row
  const Real* W;
  const int* col;
  const Real* D;
  const Real* q;
  const Real* mu;
  const Real* rho;
  // state
  Real* r;                      // AoS (npad + 1) * 3, entry npad is zero
  Real* rpli;                   // npad
  double* u;                    // AoS npad * 3 (FP64 full error output)
  // reductions and control
  double* partials;             // gridDim.x * 4
  unsigned int* barrier;        // zeroed before launch
  int* status;                  // FC3DGPU_STATUS_* bits
  double* trace;                // per-sweep incremental error
  int trace_cap;
  int trace_base;               // index of this launch's first sweep in trace
  // controls
  int max_sweeps;
  int mode;                     // 0: FP32 accelerator stop rule, 1: reference NSGS logic
  double user_tol;
  double local_tol;
  double switch_tol;
  int stall_window;
  double norm_q;
  int newton_max, pli_max, ls_max;
  int local_mode;  // one-contact solver: 0 the reference's hybrid, 1 damped Newton only (FP32 sweeps)
  // the reference's optional per-contact steps (FP64 sweeps): relaxation of
  // each new reaction with omega, and the filter of local solutions
  int relax, filter;
  double omega;
  unsigned long long spin_limit;
  unsigned long long* counters;  // optional work counters: Newton its, PLI its, line-search evals, solves, max Newton
  unsigned long long* timeline;  // optional: globaltimer at each colour phase's start and work end, per block
  int timeline_sweep;            // the sweep (1-based) the timeline records
  // bulk-copy staging of each block's slab range (one lane per contact only):
  // W, col and q of the next colour stream into dynamic shared memory while
  // the block solves the current colour; 0 bytes = off
  unsigned stage_w_bytes, stage_c_bytes, stage_q_bytes, stage_d_bytes;
  // neighbourhood synchronisation between the colours of a sweep (one lane
  // per contact only): block b waits only for the blocks whose rows share a
  // W block with its rows, nbr[nbr_ptr[b] .. nbr_ptr[b + 1]), built for a
  // grid of nbr_grid blocks; null or another grid = a grid-wide barrier
  const int* nbr_ptr;
  const int* nbr;
  int nbr_grid;
  // outputs (written by block 0, thread 0)
  double* out;                  // [0] sweeps, [1] incr, [2] full error, [3] info, [4] working tol
};

#define FC3D_PASS_SLABS 16

// Barrier flags: one per block, each on its own 128-byte line so that the
// blocks polling them do not queue on a few L2 lines.
#define FC3D_FLAG_STRIDE 32

// Phase timeline entries per (colour, block)
#define FC3D_TL_STRIDE 8
#define FC3D_BARRIER_WORDS (1024 * FC3D_FLAG_STRIDE)

// Work list of one block: the contacts of the current pass whose local
// problem is not the trivial take-off, packed densely.
template <typename Real>
struct WorkList {
  int p[FC3D_PASS_SLABS * FC3D_SLAB];
  Real q[FC3D_PASS_SLABS * FC3D_SLAB][3];
  Real ro[FC3D_PASS_SLABS * FC3D_SLAB][3];
  int count[FC3D_PASS_SLABS];
};

// Work list of the staged path: also carries each contact's diagonal block,
// mu and rho, copied from the staging buffer before it is refilled.
template <typename Real>
struct WorkListS {
  // component-major, so consecutive work items sit in consecutive banks
  int p[FC3D_PASS_SLABS * FC3D_SLAB];
  Real q[3][FC3D_PASS_SLABS * FC3D_SLAB];
  Real ro[3][FC3D_PASS_SLABS * FC3D_SLAB];
  Real m[12][FC3D_PASS_SLABS * FC3D_SLAB];  // 9 of D, mu, rhoN, rhoT
  int count[FC3D_PASS_SLABS];
};

// Slab-dataflow FP32 sweep (fc3dgpu_flow.cuh): longest slab (in slots) it
// takes, and the kernel's arguments besides SweepArgs.
#define FC3D_FLOW_MAXSLOT 16

struct FlowArgs {
  const int* dptr;     // per slab: its neighbour slabs are dep[dptr[s] .. dptr[s + 1])
  const int* dep;      // slab ids, ascending; bit 31 set: a later colour
  unsigned* done;      // per slab: neighbour-slab updates signalled to it; zero at launch
  const int2* need;    // per slab: (neighbour slabs, those of a later colour)
  double* part;        // per block: 4 slots of (sum |dr|^2, sum |r|^2)
  unsigned buf_bytes;  // shared-memory buffer of one warp
  int maxslot;         // slots of one slab the buffer holds
  const float* rec;          // per slab one record of its sweep inputs (flow_rec_floats)
  const long long* rec_off;  // float offset of slab s's record in rec
};

// Per-slab record of the FP32 inputs of a slab with ns slots, back to back:
// W (ns * 9 * 32), col (ns * 32, int), q (3 * 32), D (9 * 32), mu (32),
// rho (2 * 32); every part a 128-byte multiple, so one bulk copy stages a
// slab.  The per-warp buffer holds the record of the longest slab.
__host__ __device__ __forceinline__ unsigned flow_rec_floats(int ns) {
  return (unsigned)ns * FC3D_SLAB * (9 + 1) + FC3D_SLAB * (3 + 9 + 1 + 2);
}
__host__ __device__ __forceinline__ unsigned flow_buf_bytes(int maxslot) { return flow_rec_floats(maxslot) * 4; }

}  // namespace fc3dgpu
