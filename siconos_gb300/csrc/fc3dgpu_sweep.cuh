// Persistent coloured NSGS kernel.
//
// One cooperative launch runs every sweep of a solve: for each colour, warps
// take (slab, round) work units; T lanes own one contact, form the
// off-diagonal block-row product q_i + sum_j W_ij r_j from coalesced
// slot-major loads (fc3d_local_problem_compute_q, fc3d_local_problem_tools.c:
// 48-63, and SBM_row_prod_no_diag_3x3, SparseBlockMatrix.c:1431-1490), then
// run the local solver in registers; a bounded grid barrier separates colours
// (contacts of one colour share no body, so their W blocks are zero and the
// order inside a colour does not matter).  After the last colour the light
// error sqrt(sum |dr|^2)/|r| (fc3d_nsgs.c:80-96) is reduced in a fixed
// order, so every block takes the same decision.  In reference mode the
// kernel also evaluates fc3d_compute_error (fc3d_compute_error.c:70-122) and
// the tolerance manager (tolerance_manager.h:203-225) on the device, exactly
// when fc3d_nsgs would (fc3d_nsgs.c:496-534, :839-851, :877-895).
#pragma once
#include <cfloat>
#include <cuda_runtime.h>

#include "fc3dgpu_layout.cuh"
#include "fc3dgpu_local.cuh"

namespace fc3dgpu {

// Threads per block: 10 warps for the FP32 kernel (a block's slab range of
// up to 10 slabs is covered in one round), 8 for FP64 (its register use
// leaves room for 256 threads only).  Both give one block per SM.
template <typename Real>
struct BlockDim {
  static constexpr int value = sizeof(Real) == 4 ? 320 : 256;
};
#define FC3D_BLOCK_MAX 320
#define FC3D_RSTRIDE 4

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier with a poll limit.  Each block publishes its barrier
// count in its own flag word (a store, no contended atomic), and one warp of
// every block polls all flags with relaxed loads issued together (one memory
// round trip per poll) until each shows the count, then fences (acquire).  On
// expiry the block records FC3DGPU_STATUS_BARRIER_TIMEOUT and returns false;
// its caller leaves the kernel, and every other block then times out at its
// next barrier.  The flags must be zero at launch.
__device__ __forceinline__ bool grid_barrier(unsigned* flags, unsigned& epoch, unsigned long long limit, int* status) {
  __shared__ int s_ok;
  __syncthreads();
  epoch++;
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    if (lane == 0) st_release_u32(&flags[blockIdx.x * FC3D_FLAG_STRIDE], epoch);
    unsigned long long n = 0;
    int ok = 1;
    for (;;) {
      bool mine = true;
#pragma unroll 8
      for (int b = lane; b < (int)gridDim.x; b += 32)
        mine &= (ld_relaxed_u32(&flags[b * FC3D_FLAG_STRIDE]) >= epoch);
      if (__all_sync(0xffffffffu, mine)) break;
      if (++n > limit) {
        ok = 0;
        if (lane == 0) atomicOr(status, 1);
        break;
      }
      if (n > 256) __nanosleep(32);
    }
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    if (lane == 0) s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Arrive as the grid barrier does (flag = epoch) but wait only for the
// listed blocks.  Every block passes the same sequence of barriers, so equal
// epochs mean the same point of the sweep.  A block can then run at most one
// colour ahead of any neighbour: rows of colour c read their neighbours'
// reactions after those neighbours finished colour c - 1 and before they
// start colour c + 1, exactly as in the grid-synchronised sweep.
__device__ __forceinline__ bool nbr_barrier(unsigned* flags, unsigned& epoch, const int* nbr, int nn,
                                            unsigned long long limit, int* status) {
  __shared__ int s_ok;
  __syncthreads();
  epoch++;
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    if (lane == 0) st_release_u32(&flags[blockIdx.x * FC3D_FLAG_STRIDE], epoch);
    unsigned long long n = 0;
    int ok = 1;
    for (;;) {
      bool mine = true;
      for (int k = lane; k < nn; k += 32)
        mine &= (ld_relaxed_u32(&flags[__ldg(&nbr[k]) * FC3D_FLAG_STRIDE]) >= epoch);
      if (__all_sync(0xffffffffu, mine)) break;
      if (++n > limit) {
        ok = 0;
        if (lane == 0) atomicOr(status, 1);
        break;
      }
      if (n > 256) __nanosleep(32);
    }
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    if (lane == 0) s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

template <int N>
__device__ __forceinline__ void block_sum(double v[N], double* out_partials) {
  __shared__ double sh[FC3D_BLOCK_MAX / 32][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < N; i++) {
    double x = v[i];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sh[w][i] = x;
  }
  __syncthreads();
  if (threadIdx.x < N) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k][threadIdx.x];
    out_partials[threadIdx.x] = s;
  }
  __syncthreads();
}

// Sum slot k of every block's partials in a fixed order; every block gets
// the same value.  Called after a grid barrier.
template <int N>
__device__ __forceinline__ void grid_sum(const double* partials, int slot0, double out[N]) {
  __shared__ double res[8];
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
#pragma unroll
    for (int i = 0; i < N; i++) {
      double s = 0.0;
      for (int b = lane; b < (int)gridDim.x; b += 32) s += __ldcg(&partials[b * 8 + slot0 + i]);
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) res[i] = s;
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < N; i++) out[i] = res[i];
  __syncthreads();
}

template <typename Real>
__device__ __forceinline__ void load_r3(const Real* r, int p, Real out[3]);
template <>
__device__ __forceinline__ void load_r3<float>(const float* r, int p, float out[3]) {
  float4 v = __ldcg(reinterpret_cast<const float4*>(r) + p);
  out[0] = v.x;
  out[1] = v.y;
  out[2] = v.z;
}
template <>
__device__ __forceinline__ void load_r3<double>(const double* r, int p, double out[3]) {
  const double2* q = reinterpret_cast<const double2*>(r) + 2 * (size_t)p;
  double2 a = __ldcg(q), b = __ldcg(q + 1);
  out[0] = a.x;
  out[1] = a.y;
  out[2] = b.x;
}

// The reference's optional steps after a contact's local solve
// (fc3d_nsgs.c:760-830): the new reaction relaxed towards the old one,
// omega rn + (1 - omega) o (performRelaxation_3, :73-78; the light-error
// term then uses the relaxed reaction), and the filter that keeps the old
// reaction when the local solver's residual is not finite or above 1
// (acceptLocalReactionFiltered, :338-389).  keep: the reaction to store.
template <typename Real>
__device__ __forceinline__ void nsgs_accept(const SweepArgs<Real>& a, const LocalProblem<Real>& L, const Real o[3],
                                            Real rn[3], Real keep[3]) {
  if (a.relax) {
    const Real w = (Real)a.omega;
    rn[0] = w * rn[0] + (Real(1.0) - w) * o[0];
    rn[1] = w * rn[1] + (Real(1.0) - w) * o[1];
    rn[2] = w * rn[2] + (Real(1.0) - w) * o[2];
  }
  const bool discard = a.filter && (isnan(L.residual) || isinf(L.residual) || L.residual > Real(1.0));
  keep[0] = discard ? o[0] : rn[0];
  keep[1] = discard ? o[1] : rn[1];
  keep[2] = discard ? o[2] : rn[2];
}

// A take-off contact (local reaction 0, residual 0) under relaxation: the
// zero relaxed towards the old reaction as nsgs_accept relaxes any local
// solution, stored, with its light-error and norm terms.
template <typename Real>
__device__ __forceinline__ void takeoff_relaxed(const SweepArgs<Real>& a, const Real o[3], Real* rp, double& dr2,
                                                double& rr2) {
  const Real w = (Real)a.omega;
  Real rn[3];
  rn[0] = w * Real(0.0) + (Real(1.0) - w) * o[0];
  rn[1] = w * Real(0.0) + (Real(1.0) - w) * o[1];
  rn[2] = w * Real(0.0) + (Real(1.0) - w) * o[2];
  rp[0] = rn[0];
  rp[1] = rn[1];
  rp[2] = rn[2];
  const double d0 = (double)o[0] - (double)rn[0], d1 = (double)o[1] - (double)rn[1], d2 = (double)o[2] - (double)rn[2];
  dr2 += d0 * d0 + d1 * d1 + d2 * d2;
  rr2 += (double)rn[0] * rn[0] + (double)rn[1] * rn[1] + (double)rn[2] * rn[2];
}

template <typename Real, int T>
__device__ __forceinline__ void process_unit(const SweepArgs<Real>& a, int slab, int round, int lane, Real ltol,
                                             double& dr2, double& rr2) {
  constexpr int CPR = 32 / T;
  const int g = lane / T, j = lane % T;
  const int k = round * CPR + g;
  const int p = slab * FC3D_SLAB + k;
  const long long base = a.slab_off[slab];
  const int ns = a.slab_nslot[slab];
  const size_t qi = (size_t)slab * 3 * FC3D_SLAB + k;
  const Real q0 = a.q[qi], q1 = a.q[qi + FC3D_SLAB], q2 = a.q[qi + 2 * FC3D_SLAB];
  Real acc[3];
  if (T == 1) {
    acc[0] = q0;
    acc[1] = q1;
    acc[2] = q2;
  } else {
    acc[0] = 0;
    acc[1] = 0;
    acc[2] = 0;
  }
  // slots in chunks of CH, fully unrolled: the column indices and W
  // elements of a chunk are requested together, then the dependent r
  // gathers, so one row costs two memory round trips per chunk instead of
  // two per slot.  Accumulation stays in slot order.
  constexpr int CH = sizeof(Real) == 4 ? 8 : 4;
  for (int s0 = j; s0 < ns; s0 += CH * T) {
    int pj[CH];
    Real wv[CH][9];
#pragma unroll
    for (int c = 0; c < CH; c++) {
      const int s = s0 + c * T;
      const size_t sl = (size_t)(base + (s < ns ? s : 0));
      pj[c] = s < ns ? __ldg(&a.col[sl * FC3D_SLAB + k]) : a.npad;
      const Real* w = a.W + sl * 9 * FC3D_SLAB + k;
#pragma unroll
      for (int e = 0; e < 9; e++) wv[c][e] = s < ns ? __ldg(&w[e * FC3D_SLAB]) : Real(0);
    }
    Real rv[CH][3];
#pragma unroll
    for (int c = 0; c < CH; c++) load_r3<Real>(a.r, pj[c], rv[c]);
#pragma unroll
    for (int c = 0; c < CH; c++)
      if (s0 + c * T < ns) mvp3x3(wv[c], rv[c], acc);
  }
  if (T > 1) {
#pragma unroll
    for (int o = T / 2; o >= 1; o >>= 1) {
      acc[0] += __shfl_xor_sync(0xffffffffu, acc[0], o);
      acc[1] += __shfl_xor_sync(0xffffffffu, acc[1], o);
      acc[2] += __shfl_xor_sync(0xffffffffu, acc[2], o);
    }
    acc[0] = q0 + acc[0];
    acc[1] = q1 + acc[1];
    acc[2] = q2 + acc[2];
  }
  if (__ldg(&a.perm[p]) < 0) return;
  LocalProblem<Real> L;
#pragma unroll
  for (int e = 0; e < 9; e++) L.M[e] = __ldg(&a.D[((size_t)slab * 9 + e) * FC3D_SLAB + k]);
  L.q[0] = acc[0];
  L.q[1] = acc[1];
  L.q[2] = acc[2];
  L.mu = __ldg(&a.mu[(size_t)slab * FC3D_SLAB + k]);
  L.rhoN = __ldg(&a.rho[((size_t)slab * 2) * FC3D_SLAB + k]);
  L.rhoT = __ldg(&a.rho[((size_t)slab * 2 + 1) * FC3D_SLAB + k]);
  L.rho_pli = a.rpli[p];
  L.tol = ltol;
  L.newton_max = a.newton_max;
  L.pli_max = a.pli_max;
  L.ls_max = a.ls_max;
  L.mode = a.local_mode;
  L.n_newton = 0;
  L.n_pli = 0;
  L.n_ls = 0;
  Real ro[3], rn[3];
  load_r3<Real>(a.r, p, ro);
  rn[0] = ro[0];
  rn[1] = ro[1];
  rn[2] = ro[2];
  local_solve(L, rn);
  Real keep[3];
  nsgs_accept(a, L, ro, rn, keep);
  if (a.counters) {
    // warp-aggregated: one atomic per counter per warp and unit
    unsigned long long c0 = j == 0 ? L.n_newton : 0, c1 = j == 0 ? L.n_pli : 0, c2 = j == 0 ? L.n_ls : 0;
    unsigned long long c4 = j == 0 ? L.n_newton : 0;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      c0 += __shfl_xor_sync(__activemask(), c0, o);
      c1 += __shfl_xor_sync(__activemask(), c1, o);
      c2 += __shfl_xor_sync(__activemask(), c2, o);
      c4 = max(c4, __shfl_xor_sync(__activemask(), c4, o));
    }
    if (lane == (__ffs(__activemask()) - 1)) {
      atomicAdd(&a.counters[0], c0);
      atomicAdd(&a.counters[1], c1);
      atomicAdd(&a.counters[2], c2);
      atomicAdd(&a.counters[3], (unsigned long long)__popc(__activemask()) / T);
      atomicMax(&a.counters[4], c4);
    }
  }
  if (j == 0) {
    Real* rp = a.r + (size_t)p * FC3D_RSTRIDE;
    rp[0] = keep[0];
    rp[1] = keep[1];
    rp[2] = keep[2];
    a.rpli[p] = L.rho_pli;
    const double d0 = (double)ro[0] - (double)rn[0], d1 = (double)ro[1] - (double)rn[1],
                 d2 = (double)ro[2] - (double)rn[2];
    dr2 += d0 * d0 + d1 * d1 + d2 * d2;
    rr2 += (double)keep[0] * keep[0] + (double)keep[1] * keep[1] + (double)keep[2] * keep[2];
  }
}

// ---- bulk copies (TMA engine, non-tensor) into shared memory -------------
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// global -> shared bulk copy completing on an mbarrier; 16-byte aligned
// addresses, size a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Polls granted to the wait for a block's own bulk copies in flight before
// it leaves the kernel (however small the spin limit of the other waits:
// no block exits with a copy into its shared memory still running).
#define FC3D_EXIT_WAIT (1ULL << 24)

__device__ __forceinline__ unsigned long long exit_wait_limit(unsigned long long spin_limit) {
  return spin_limit > FC3D_EXIT_WAIT ? spin_limit : FC3D_EXIT_WAIT;
}

// Bounded wait for the staging barrier: on expiry records the timeout bit.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity, unsigned long long limit,
                                                  int* status) {
  unsigned long long n = 0;
  while (!mbar_try_wait(bar, parity)) {
    if (++n > limit) {
      atomicOr(status, 1);
      return false;
    }
  }
  return true;
}

template <typename Real>
__device__ __forceinline__ void solve_item(const SweepArgs<Real>& a, WorkList<Real>& wk, int t, Real ltol, double& dr2,
                                           double& rr2) {
  const int pp = wk.p[t];
  const int sl = pp / FC3D_SLAB, k = pp % FC3D_SLAB;
  LocalProblem<Real> L;
#pragma unroll
  for (int e = 0; e < 9; e++) L.M[e] = __ldg(&a.D[((size_t)sl * 9 + e) * FC3D_SLAB + k]);
  L.q[0] = wk.q[t][0];
  L.q[1] = wk.q[t][1];
  L.q[2] = wk.q[t][2];
  L.mu = __ldg(&a.mu[(size_t)sl * FC3D_SLAB + k]);
  L.rhoN = __ldg(&a.rho[((size_t)sl * 2) * FC3D_SLAB + k]);
  L.rhoT = __ldg(&a.rho[((size_t)sl * 2 + 1) * FC3D_SLAB + k]);
  L.rho_pli = __ldcg(&a.rpli[pp]);
  L.tol = ltol;
  L.newton_max = a.newton_max;
  L.pli_max = a.pli_max;
  L.ls_max = a.ls_max;
  L.mode = a.local_mode;
  L.n_newton = 0;
  L.n_pli = 0;
  L.n_ls = 0;
  Real o[3] = {wk.ro[t][0], wk.ro[t][1], wk.ro[t][2]};
  Real rn[3] = {o[0], o[1], o[2]};
  local_solve(L, rn);
  Real keep[3];
  nsgs_accept(a, L, o, rn, keep);
  Real* rp = a.r + (size_t)pp * FC3D_RSTRIDE;
  rp[0] = keep[0];
  rp[1] = keep[1];
  rp[2] = keep[2];
  a.rpli[pp] = L.rho_pli;
  const double d0 = (double)o[0] - (double)rn[0], d1 = (double)o[1] - (double)rn[1], d2 = (double)o[2] - (double)rn[2];
  dr2 += d0 * d0 + d1 * d1 + d2 * d2;
  rr2 += (double)keep[0] * keep[0] + (double)keep[1] * keep[1] + (double)keep[2] * keep[2];
  if (a.counters) {
    atomicAdd(&a.counters[0], (unsigned long long)L.n_newton);
    atomicAdd(&a.counters[1], (unsigned long long)L.n_pli);
    atomicAdd(&a.counters[2], (unsigned long long)L.n_ls);
    atomicAdd(&a.counters[3], 1ULL);
    atomicMax(&a.counters[4], (unsigned long long)L.n_newton);
  }
}

// Slab range [lo, hi) of one colour handled by this block.
__device__ __forceinline__ void block_range(int s0, int s1, int& lo, int& hi) {
  const int n = s1 - s0;
  lo = s0 + (int)((long long)n * blockIdx.x / gridDim.x);
  hi = s0 + (int)((long long)n * (blockIdx.x + 1) / gridDim.x);
}

// One colour with one lane per contact.  The colour's slabs are split into
// one contiguous range per block (so no block takes a second round while
// others idle) and a block handles its range in passes of up to
// FC3D_PASS_SLABS slabs.  Every lane forms its contact's local q in the
// reference's slot order.  A contact with q_n > -eps is the trivial take-off
// of the local solver (onecontact.c:234-245): r = 0, finished at once.  The
// others are packed in slab order (ballot + fixed prefix, so the packing is
// deterministic) and solved by the first threads of the block: one local
// solve latency per pass, with lanes busy instead of idling beside
// take-offs.
template <typename Real>
__device__ __forceinline__ void process_range_compact(const SweepArgs<Real>& a, int lo, int hi, Real ltol,
                                                      double& dr2, double& rr2, WorkList<Real>& wk,
                                                      unsigned long long* tl) {
  constexpr int NWB = BlockDim<Real>::value / 32;
  constexpr int MAXR = (FC3D_PASS_SLABS + NWB - 1) / NWB;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int ps = lo; ps < hi; ps += FC3D_PASS_SLABS) {
    const int np = min(FC3D_PASS_SLABS, hi - ps);
    Real acc[MAXR][3], ro[MAXR][3];
    unsigned msk[MAXR];
#pragma unroll
    for (int j = 0; j < MAXR; j++) {
      const int i = w + j * NWB;
      msk[j] = 0;
      if (i < np) {
        const int slab = ps + i;
        const int p = slab * FC3D_SLAB + lane;
        bool work = false;
        acc[j][0] = acc[j][1] = acc[j][2] = 0;
        ro[j][0] = ro[j][1] = ro[j][2] = 0;
        if (__ldg(&a.perm[p]) >= 0) {
          const long long base = a.slab_off[slab];
          const int ns = a.slab_nslot[slab];
          const size_t qi = (size_t)slab * 3 * FC3D_SLAB + lane;
          acc[j][0] = a.q[qi];
          acc[j][1] = a.q[qi + FC3D_SLAB];
          acc[j][2] = a.q[qi + 2 * FC3D_SLAB];
          constexpr int CH = sizeof(Real) == 4 ? 8 : 4;
          for (int t0 = 0; t0 < ns; t0 += CH) {
            int pj[CH];
            Real wv[CH][9];
#pragma unroll
            for (int c = 0; c < CH; c++) {
              const int sidx = t0 + c;
              const size_t sl = (size_t)(base + (sidx < ns ? sidx : 0));
              pj[c] = sidx < ns ? __ldg(&a.col[sl * FC3D_SLAB + lane]) : a.npad;
              const Real* wp = a.W + sl * 9 * FC3D_SLAB + lane;
#pragma unroll
              for (int e = 0; e < 9; e++) wv[c][e] = sidx < ns ? __ldg(&wp[e * FC3D_SLAB]) : Real(0);
            }
            Real rv[CH][3];
#pragma unroll
            for (int c = 0; c < CH; c++) load_r3<Real>(a.r, pj[c], rv[c]);
#pragma unroll
            for (int c = 0; c < CH; c++)
              if (t0 + c < ns) mvp3x3(wv[c], rv[c], acc[j]);
          }
          load_r3<Real>(a.r, p, ro[j]);
          if (acc[j][0] > -Eps<Real>::v()) {
            Real* rp = a.r + (size_t)p * FC3D_RSTRIDE;
            if (a.relax) {
              takeoff_relaxed(a, ro[j], rp, dr2, rr2);
            } else {
              rp[0] = 0;
              rp[1] = 0;
              rp[2] = 0;
              dr2 += (double)ro[j][0] * ro[j][0] + (double)ro[j][1] * ro[j][1] + (double)ro[j][2] * ro[j][2];
            }
          } else {
            work = true;
          }
        }
        msk[j] = __ballot_sync(0xffffffffu, work);
        if (lane == 0) wk.count[i] = __popc(msk[j]);
      }
    }
    __syncthreads();
    int total = 0;
    for (int k = 0; k < np; k++) total += wk.count[k];
    if (tl && threadIdx.x == 0) {
      tl[0] = globaltimer_ns();
      tl[1] = (unsigned long long)total;
    }
#pragma unroll
    for (int j = 0; j < MAXR; j++) {
      const int i = w + j * NWB;
      if (i < np && (msk[j] >> lane) & 1u) {
        int off = 0;
        for (int k = 0; k < i; k++) off += wk.count[k];
        const int idx = off + __popc(msk[j] & ((1u << lane) - 1));
        wk.p[idx] = (ps + i) * FC3D_SLAB + lane;
        wk.q[idx][0] = acc[j][0];
        wk.q[idx][1] = acc[j][1];
        wk.q[idx][2] = acc[j][2];
        wk.ro[idx][0] = ro[j][0];
        wk.ro[idx][1] = ro[j][1];
        wk.ro[idx][2] = ro[j][2];
      }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < total; t += blockDim.x) solve_item(a, wk, t, ltol, dr2, rr2);
    __syncthreads();
  }
}

// Issue the bulk copies of W, col and q for slabs [lo, hi) into the
// staging buffers (one thread).  The caller made sure the previous
// contents were consumed (block barrier + proxy fence).
// Slot range [o0, o0 + slots) of the slab range [lo, hi).
template <typename Real>
__device__ __forceinline__ void range_slots(const SweepArgs<Real>& a, int lo, int hi, long long& o0,
                                            long long& slots) {
  o0 = a.slab_off[lo];
  slots = (hi < a.nslab ? a.slab_off[hi] : a.slab_off[hi - 1] + a.slab_nslot[hi - 1]) - o0;
}

template <typename Real>
__device__ __forceinline__ void stage_issue(const SweepArgs<Real>& a, int lo, int hi, unsigned char* stage,
                                            unsigned long long* bar, long long o0 = -1, long long slots = 0) {
  if (o0 < 0) range_slots(a, lo, hi, o0, slots);
  const unsigned wb = (unsigned)(slots * 9 * FC3D_SLAB * sizeof(Real));
  const unsigned cb = (unsigned)(slots * FC3D_SLAB * sizeof(int));
  const unsigned qb = (unsigned)((hi - lo) * 3 * FC3D_SLAB * sizeof(Real));
  const unsigned db = (unsigned)((hi - lo) * 9 * FC3D_SLAB * sizeof(Real));
  const unsigned mb = (unsigned)((hi - lo) * FC3D_SLAB * sizeof(Real));
  const unsigned rb = 2 * mb;
  unsigned char* sq = stage + a.stage_w_bytes + a.stage_c_bytes;
  unsigned char* sd = sq + a.stage_q_bytes;
  unsigned char* sm = sd + a.stage_d_bytes;
  unsigned char* sr = sm + a.stage_d_bytes / 9;
  mbar_arrive_expect_tx(bar, wb + cb + qb + db + mb + rb);
  if (wb) bulk_g2s(stage, a.W + (size_t)o0 * 9 * FC3D_SLAB, wb, bar);
  if (cb) bulk_g2s(stage + a.stage_w_bytes, a.col + (size_t)o0 * FC3D_SLAB, cb, bar);
  bulk_g2s(sq, a.q + (size_t)lo * 3 * FC3D_SLAB, qb, bar);
  bulk_g2s(sd, a.D + (size_t)lo * 9 * FC3D_SLAB, db, bar);
  bulk_g2s(sm, a.mu + (size_t)lo * FC3D_SLAB, mb, bar);
  bulk_g2s(sr, a.rho + (size_t)lo * 2 * FC3D_SLAB, rb, bar);
}

// process_colour_compact with W, col and q read from the staged shared
// memory copy of the block's range (which must fit one pass), and the next
// colour's range staged as soon as this one's row products are done.
// Local solve of row pp from L's diagonal block, q, mu and rho (set by the
// caller) and the reaction o before it; writes the new reaction.
template <typename Real>
__device__ __forceinline__ void solve_row_s(const SweepArgs<Real>& a, LocalProblem<Real>& L, int pp, const Real o[3],
                                            Real ltol, double& dr2, double& rr2) {
  L.rho_pli = __ldcg(&a.rpli[pp]);
  L.tol = ltol;
  L.newton_max = a.newton_max;
  L.pli_max = a.pli_max;
  L.ls_max = a.ls_max;
  L.mode = a.local_mode;
  L.n_newton = 0;
  L.n_pli = 0;
  L.n_ls = 0;
  Real rn[3] = {o[0], o[1], o[2]};
  local_solve(L, rn);
  Real keep[3];
  nsgs_accept(a, L, o, rn, keep);
  Real* rp = a.r + (size_t)pp * FC3D_RSTRIDE;
  rp[0] = keep[0];
  rp[1] = keep[1];
  rp[2] = keep[2];
  a.rpli[pp] = L.rho_pli;
  const double d0 = (double)o[0] - (double)rn[0], d1 = (double)o[1] - (double)rn[1], d2 = (double)o[2] - (double)rn[2];
  dr2 += d0 * d0 + d1 * d1 + d2 * d2;
  rr2 += (double)keep[0] * keep[0] + (double)keep[1] * keep[1] + (double)keep[2] * keep[2];
  if (a.counters) {
    atomicAdd(&a.counters[0], (unsigned long long)L.n_newton);
    atomicAdd(&a.counters[1], (unsigned long long)L.n_pli);
    atomicAdd(&a.counters[2], (unsigned long long)L.n_ls);
    atomicAdd(&a.counters[3], 1ULL);
    atomicMax(&a.counters[4], (unsigned long long)L.n_newton);
  }
}

template <typename Real>
__device__ __forceinline__ void solve_item_s(const SweepArgs<Real>& a, WorkListS<Real>& wk, int t, Real ltol,
                                             double& dr2, double& rr2) {
  LocalProblem<Real> L;
#pragma unroll
  for (int e = 0; e < 9; e++) L.M[e] = wk.m[e][t];
  L.q[0] = wk.q[0][t];
  L.q[1] = wk.q[1][t];
  L.q[2] = wk.q[2][t];
  L.mu = wk.m[9][t];
  L.rhoN = wk.m[10][t];
  L.rhoT = wk.m[11][t];
  const Real o[3] = {wk.ro[0][t], wk.ro[1][t], wk.ro[2][t]};
  solve_row_s(a, L, wk.p[t], o, ltol, dr2, rr2);
}

// process_colour_compact with every per-slab input (W, col, q, D, mu, rho)
// read from the staged shared-memory copy of the block's range (which must
// fit one pass).  The only global reads left in the row product are the
// neighbour and own reactions, all issued together.  The next colour's
// range is staged as soon as this one's inputs have been copied out, so it
// streams in while this colour is solved and the grid waits.
template <typename Real>
__device__ __forceinline__ bool process_colour_staged(const SweepArgs<Real>& a, int c, Real ltol, double& dr2,
                                                      double& rr2, WorkListS<Real>& wk, unsigned char* stage,
                                                      unsigned long long* bar, unsigned& parity, bool& pending,
                                                      unsigned long long* tl) {
  constexpr int NWB = BlockDim<Real>::value / 32;
  constexpr int MAXR = (FC3D_PASS_SLABS + NWB - 1) / NWB;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int lo, hi;
  block_range(a.sptr[c], a.sptr[c + 1], lo, hi);
  const int np = hi - lo;
  const int cn = (c + 1 < a.ncol) ? c + 1 : 0;
  int nlo, nhi;
  block_range(a.sptr[cn], a.sptr[cn + 1], nlo, nhi);
  if (np > 0) {
    const int first_row = a.sptr[c] * FC3D_SLAB, end_row = first_row + a.ccount[c];
    // independent global loads first: slab metadata and own reactions
    long long off[MAXR];
    int nsl[MAXR];
    Real ro[MAXR][3];
#pragma unroll
    for (int j = 0; j < MAXR; j++) {
      const int i = w + j * NWB;
      off[j] = 0;
      nsl[j] = 0;
      ro[j][0] = ro[j][1] = ro[j][2] = 0;
      if (i < np) {
        const int slab = lo + i;
        off[j] = a.slab_off[slab];
        nsl[j] = a.slab_nslot[slab];
        const int p = slab * FC3D_SLAB + lane;
        if (p < end_row) load_r3<Real>(a.r, p, ro[j]);
      }
    }
    const long long o0 = a.slab_off[lo];
    // the last thread stages the next colour (it rarely has a local solve,
    // so the copy's set-up does not delay one); its slot range is read now
    const bool issuer = threadIdx.x == blockDim.x - 1;
    long long n_o0 = -1, n_slots = 0;
    if (issuer && nhi > nlo) range_slots(a, nlo, nhi, n_o0, n_slots);
    if (pending) {
      if (!mbar_wait_bounded(bar, parity, a.spin_limit, a.status)) return false;
      parity ^= 1u;
      pending = false;
    }
    if (tl && threadIdx.x == 0) tl[2] = globaltimer_ns();
    const Real* Ws = reinterpret_cast<const Real*>(stage);
    const int* Cs = reinterpret_cast<const int*>(stage + a.stage_w_bytes);
    const Real* Qs = reinterpret_cast<const Real*>(stage + a.stage_w_bytes + a.stage_c_bytes);
    const Real* Ds = reinterpret_cast<const Real*>(stage + a.stage_w_bytes + a.stage_c_bytes + a.stage_q_bytes);
    const Real* Ms = Ds + a.stage_d_bytes / sizeof(Real) / 9 * 9;
    const Real* Rs = Ms + a.stage_d_bytes / sizeof(Real) / 9;
    Real acc[MAXR][3];
    unsigned msk[MAXR];
#pragma unroll
    for (int j = 0; j < MAXR; j++) {
      const int i = w + j * NWB;
      msk[j] = 0;
      if (i < np) {
        const int slab = lo + i;
        const int p = slab * FC3D_SLAB + lane;
        bool work = false;
        acc[j][0] = acc[j][1] = acc[j][2] = 0;
        if (p < end_row) {
          const int rel = (int)(off[j] - o0);
          const int ns = nsl[j];
          acc[j][0] = Qs[(i * 3 + 0) * FC3D_SLAB + lane];
          acc[j][1] = Qs[(i * 3 + 1) * FC3D_SLAB + lane];
          acc[j][2] = Qs[(i * 3 + 2) * FC3D_SLAB + lane];
          constexpr int CH = 16;
          for (int t0 = 0; t0 < ns; t0 += CH) {
            Real rv[CH][3];
#pragma unroll
            for (int k = 0; k < CH; k++) {
              const int pj = t0 + k < ns ? Cs[(rel + t0 + k) * FC3D_SLAB + lane] : a.npad;
              load_r3<Real>(a.r, pj, rv[k]);
            }
#pragma unroll
            for (int k = 0; k < CH; k++) {
              if (t0 + k < ns) {
                const Real* wp = Ws + (size_t)(rel + t0 + k) * 9 * FC3D_SLAB + lane;
                Real wv[9];
#pragma unroll
                for (int e = 0; e < 9; e++) wv[e] = wp[e * FC3D_SLAB];
                mvp3x3(wv, rv[k], acc[j]);
              }
            }
          }
          if (acc[j][0] > -Eps<Real>::v()) {
            Real* rp = a.r + (size_t)p * FC3D_RSTRIDE;
            if (a.relax) {
              takeoff_relaxed(a, ro[j], rp, dr2, rr2);
            } else {
              rp[0] = 0;
              rp[1] = 0;
              rp[2] = 0;
              dr2 += (double)ro[j][0] * ro[j][0] + (double)ro[j][1] * ro[j][1] + (double)ro[j][2] * ro[j][2];
            }
          } else {
            work = true;
          }
        }
        msk[j] = __ballot_sync(0xffffffffu, work);
        if (lane == 0) wk.count[i] = __popc(msk[j]);
      }
      if (j == 0 && tl && threadIdx.x == 0) tl[3] = globaltimer_ns();
    }
    if (np <= NWB) {
      // one slab per warp: every lane solves its own row where it sits, with
      // no compaction through the work list (a block has at most one row
      // per thread either way)
      const bool work = w < np && ((msk[0] >> lane) & 1u);
      LocalProblem<Real> L;
      if (work) {
#pragma unroll
        for (int e = 0; e < 9; e++) L.M[e] = Ds[(w * 9 + e) * FC3D_SLAB + lane];
        L.mu = Ms[w * FC3D_SLAB + lane];
        L.rhoN = Rs[(w * 2) * FC3D_SLAB + lane];
        L.rhoT = Rs[(w * 2 + 1) * FC3D_SLAB + lane];
        L.q[0] = acc[0][0];
        L.q[1] = acc[0][1];
        L.q[2] = acc[0][2];
      }
      __syncthreads();
      // every input of this range read: stage the next colour's range
      if (issuer && nhi > nlo) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        stage_issue(a, nlo, nhi, stage, bar, n_o0, n_slots);
      }
      if (nhi > nlo) pending = true;
      if (tl && threadIdx.x == 0) {
        int total = 0;
        for (int k = 0; k < np; k++) total += wk.count[k];
        tl[0] = globaltimer_ns();
        tl[1] = (unsigned long long)total;
      }
      if (work) solve_row_s(a, L, (lo + w) * FC3D_SLAB + lane, ro[0], ltol, dr2, rr2);
      return true;
    }
    __syncthreads();
    int total = 0;
    for (int k = 0; k < np; k++) total += wk.count[k];
#pragma unroll
    for (int j = 0; j < MAXR; j++) {
      const int i = w + j * NWB;
      if (i < np && (msk[j] >> lane) & 1u) {
        int o = 0;
        for (int k = 0; k < i; k++) o += wk.count[k];
        const int idx = o + __popc(msk[j] & ((1u << lane) - 1));
        wk.p[idx] = (lo + i) * FC3D_SLAB + lane;
        wk.q[0][idx] = acc[j][0];
        wk.q[1][idx] = acc[j][1];
        wk.q[2][idx] = acc[j][2];
        wk.ro[0][idx] = ro[j][0];
        wk.ro[1][idx] = ro[j][1];
        wk.ro[2][idx] = ro[j][2];
#pragma unroll
        for (int e = 0; e < 9; e++) wk.m[e][idx] = Ds[(i * 9 + e) * FC3D_SLAB + lane];
        wk.m[9][idx] = Ms[i * FC3D_SLAB + lane];
        wk.m[10][idx] = Rs[(i * 2) * FC3D_SLAB + lane];
        wk.m[11][idx] = Rs[(i * 2 + 1) * FC3D_SLAB + lane];
      }
    }
    __syncthreads();
    // every input of this range copied out: stage the next colour's range
    if (issuer && nhi > nlo) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      stage_issue(a, nlo, nhi, stage, bar, n_o0, n_slots);
    }
    if (nhi > nlo) pending = true;
    if (tl && threadIdx.x == 0) {
      tl[0] = globaltimer_ns();
      tl[1] = (unsigned long long)total;
    }
    for (int t = threadIdx.x; t < total; t += blockDim.x) solve_item_s(a, wk, t, ltol, dr2, rr2);
    __syncthreads();
  } else if (nhi > nlo && !pending) {
    // nothing to do in this colour; stage the next one (buffer is free)
    if (threadIdx.x == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      stage_issue(a, nlo, nhi, stage, bar);
    }
    pending = true;
  }
  return true;
}

// u = q + W r for every row in CSR block order (diagonal at its own slot
// position, SBM_gemv_3x3, SparseBlockMatrix.c:360-419) and the partial sums
// of the squared natural-map error, |u|^2 and |r|^2.  FP64 only.
template <typename Real>
__device__ __forceinline__ void full_error_rows(const SweepArgs<Real>& a, double v[3], int p0 = 0, int p1 = -1,
                                                int tid = -1, int nth = -1) {
  v[0] = v[1] = v[2] = 0.0;
  if (p1 < 0) p1 = a.npad;
  if (tid < 0) {
    tid = blockIdx.x * blockDim.x + threadIdx.x;
    nth = gridDim.x * blockDim.x;
  }
  for (int p = p0 + tid; p < p1; p += nth) {
    if (__ldg(&a.perm[p]) < 0) continue;
    const int slab = p / FC3D_SLAB, k = p % FC3D_SLAB;
    const long long base = a.slab_off[slab];
    const int ns = a.slab_nslot[slab];
    const int dp = __ldg(&a.dpos[p]);
    const size_t qi = (size_t)slab * 3 * FC3D_SLAB + k;
    Real u[3] = {a.q[qi], a.q[qi + FC3D_SLAB], a.q[qi + 2 * FC3D_SLAB]};
    Real rp[3], D[9];
    load_r3<Real>(a.r, p, rp);
#pragma unroll
    for (int e = 0; e < 9; e++) D[e] = __ldg(&a.D[((size_t)slab * 9 + e) * FC3D_SLAB + k]);
    for (int s = 0; s < ns; s++) {
      if (s == dp) mvp3x3(D, rp, u);
      const size_t sl = (size_t)(base + s);
      const int pj = __ldg(&a.col[sl * FC3D_SLAB + k]);
      const Real* w = a.W + sl * 9 * FC3D_SLAB + k;
      Real wv[9], rv[3];
#pragma unroll
      for (int e = 0; e < 9; e++) wv[e] = __ldg(&w[e * FC3D_SLAB]);
      load_r3<Real>(a.r, pj, rv);
      mvp3x3(wv, rv, u);
    }
    if (dp >= ns) mvp3x3(D, rp, u);
    const Real mu = __ldg(&a.mu[(size_t)slab * FC3D_SLAB + k]);
    v[0] += (double)unitary_error2(rp, u, mu);
    v[1] += (double)u[0] * u[0] + (double)u[1] * u[1] + (double)u[2] * u[2];
    v[2] += (double)rp[0] * rp[0] + (double)rp[1] * rp[1] + (double)rp[2] * rp[2];
    if (a.u) {
      a.u[3 * (size_t)p + 0] = u[0];
      a.u[3 * (size_t)p + 1] = u[1];
      a.u[3 * (size_t)p + 2] = u[2];
    }
  }
}

template <typename Real>
__device__ __forceinline__ bool full_error_phase(const SweepArgs<Real>& a, int slot0, unsigned& epoch,
                                                 double& full) {
  double v[3];
  full_error_rows(a, v);
  block_sum<3>(v, a.partials + blockIdx.x * 8 + slot0);
  if (!grid_barrier(a.barrier, epoch, a.spin_limit, a.status)) return false;
  double s[3];
  grid_sum<3>(a.partials, slot0, s);
  double e = sqrt(s[0]);
  const double scal = fmax(a.norm_q, fmax(sqrt(s[2]), sqrt(s[1])));
  if (fabs(scal) > DBL_EPSILON) e /= scal;
  full = e;
  return true;
}

template <typename Real, int T>
__global__ void __launch_bounds__(BlockDim<Real>::value, 1) nsgs_kernel(const SweepArgs<Real> a) {
  __shared__ WorkList<Real> wk;
  __shared__ __align__(8) unsigned long long stage_bar;

  extern __shared__ __align__(128) unsigned char stage[];
  constexpr bool can_stage = (sizeof(Real) == 4) && T == 1;
  const bool staged = can_stage && a.stage_w_bytes > 0;
  unsigned parity = 0;
  bool pending = false;
  if (staged) {
    if (threadIdx.x == 0) {
      mbar_init(&stage_bar, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    int lo, hi;
    block_range(a.sptr[0], a.sptr[1], lo, hi);
    if (hi > lo) {
      if (threadIdx.x == 0) stage_issue(a, lo, hi, stage, &stage_bar);
      pending = true;
    }
  }
  const int lane = threadIdx.x & 31;
  const int nwb = blockDim.x >> 5;
  const int gw = blockIdx.x * nwb + (threadIdx.x >> 5), tw = gridDim.x * nwb;
  const bool local_sync = T == 1 && a.nbr_ptr != nullptr && a.nbr_grid == (int)gridDim.x;
  unsigned epoch = 0;
  double working = a.mode == 1 ? a.user_tol : fmax(a.user_tol, a.switch_tol), local_tol = a.local_tol;
  double incr = INFINITY, full = INFINITY, best = INFINITY;
  int sweep = 0, best_sweep = 0;
  bool converged = false;
  while (sweep < a.max_sweeps) {
    sweep++;
    double acc[2] = {0.0, 0.0};
    for (int c = 0; c < a.ncol; c++) {
      const int s0 = a.sptr[c], nunits = (a.sptr[c + 1] - s0) * T;
      const bool tl = a.timeline && sweep == a.timeline_sweep && threadIdx.x == 0;
      if (tl) {
        unsigned long long* e = a.timeline + ((size_t)c * gridDim.x + blockIdx.x) * FC3D_TL_STRIDE;
        e[0] = globaltimer_ns();
        e[2] = e[3] = e[4] = e[5] = e[6] = e[7] = 0;
      }
      if (can_stage && staged) {
        // the staged work list lives in dynamic shared memory after the
        // staging buffers (W, col, q, D, mu, rho)
        WorkListS<Real>& wks = *reinterpret_cast<WorkListS<Real>*>(
            stage + ((a.stage_w_bytes + a.stage_c_bytes + a.stage_q_bytes + a.stage_d_bytes / 9 * 12 + 15) & ~15u));
        if (!process_colour_staged<Real>(a, c, (Real)local_tol, acc[0], acc[1], wks, stage, &stage_bar, parity,
                                         pending,
                                         tl ? a.timeline + ((size_t)c * gridDim.x + blockIdx.x) * FC3D_TL_STRIDE + 2 : nullptr)) {
          // the staged copy the wait gave up on lands before the block leaves
          if (pending) mbar_wait_bounded(&stage_bar, parity, exit_wait_limit(a.spin_limit), a.status);
          return;
        }
      } else if (T == 1) {
        int lo, hi;
        block_range(s0, a.sptr[c + 1], lo, hi);
        process_range_compact<Real>(a, lo, hi, (Real)local_tol, acc[0], acc[1], wk,
                                    tl ? a.timeline + ((size_t)c * gridDim.x + blockIdx.x) * FC3D_TL_STRIDE + 2 : nullptr);
      } else {
        for (int u = gw; u < nunits; u += tw) {
          const long long t0 = a.counters ? clock64() : 0;
          process_unit<Real, T>(a, s0 + u / T, u % T, lane, (Real)local_tol, acc[0], acc[1]);
          if (a.counters) {
            __syncwarp();
            if (lane == 0) {
              const unsigned long long dt = (unsigned long long)(clock64() - t0);
              atomicAdd(&a.counters[5], dt);
              atomicMax(&a.counters[6], dt);
              atomicAdd(&a.counters[7], 1ULL);
            }
          }
        }
      }
      if (c == a.ncol - 1) block_sum<2>(acc, a.partials + blockIdx.x * 8);
      if (tl) a.timeline[((size_t)c * gridDim.x + blockIdx.x) * FC3D_TL_STRIDE + 1] = globaltimer_ns();
      const bool ok = (local_sync && c < a.ncol - 1)
                          ? nbr_barrier(a.barrier, epoch, a.nbr + a.nbr_ptr[blockIdx.x],
                                        a.nbr_ptr[blockIdx.x + 1] - a.nbr_ptr[blockIdx.x], a.spin_limit, a.status)
                          : grid_barrier(a.barrier, epoch, a.spin_limit, a.status);
      if (!ok) {
        if (pending) mbar_wait_bounded(&stage_bar, parity, exit_wait_limit(a.spin_limit), a.status);
        return;
      }
    }
    double s[2];
    grid_sum<2>(a.partials, 0, s);
    incr = sqrt(s[0]);
    const double nr = sqrt(s[1]);
    if (fabs(nr) > DBL_EPSILON) incr /= nr;
    if (a.trace && blockIdx.x == 0 && threadIdx.x == 0 && a.trace_base + sweep - 1 < a.trace_cap)
      a.trace[a.trace_base + sweep - 1] = incr;
    bool stop = false;
    if (a.mode == 1) {
      // check_convergence_with_adaptation (fc3d_nsgs.c:496-534)
      if (incr < working) {
        if (!full_error_phase(a, 2, epoch, full)) {
          if (pending) mbar_wait_bounded(&stage_bar, parity, exit_wait_limit(a.spin_limit), a.status);
          return;
        }
        if (full <= a.user_tol) {
          converged = true;
          stop = true;
        } else if (incr < 1e-15 || incr < DBL_EPSILON * 100.0) {
          local_tol = fmax(local_tol / 100.0, DBL_EPSILON * 1e-6);
        } else if (full > 0.0 && incr > 0.0) {
          double nt = (incr / full) * a.user_tol;
          const double user_min = a.user_tol * 1e-6, floor_tol = DBL_EPSILON * 1e-6;
          const double mint = user_min > floor_tol ? user_min : floor_tol;
          if (nt < mint) nt = mint;
          if (nt > 0.0 && nt < working) working = nt;
        }
        if (!(working > 0.0)) stop = true;
      }
    } else {
      if (!(incr == incr)) {
        if (threadIdx.x == 0) atomicOr(a.status, 2);
        stop = true;
      }
      if (incr < a.switch_tol) stop = true;
      if (incr < 0.99 * best) {
        best = incr;
        best_sweep = sweep;
      } else if (a.stall_window > 0 && sweep - best_sweep >= a.stall_window) {
        stop = true;
      }
      // the reference's adaptive convergence test on this precision's
      // iterate, against max(tol, switch_tol): the FP32 sweeps end as soon
      // as their full error (FP32 arithmetic, FP64 sums) reaches it
      if (!stop && incr < working) {
        if (!full_error_phase(a, 2, epoch, full)) {
          if (pending) mbar_wait_bounded(&stage_bar, parity, exit_wait_limit(a.spin_limit), a.status);
          return;
        }
        const double target = fmax(a.user_tol, a.switch_tol);
        if (full <= target) {
          converged = true;
          stop = true;
        } else if (full > 0.0 && incr > 0.0) {
          double nt = (incr / full) * target;
          const double mint = fmax(target * 1e-6, DBL_EPSILON * 1e-6);
          if (nt < mint) nt = mint;
          if (nt < working) working = nt;
        }
      }
    }
    if (stop) break;
  }
  if (pending) {
    // a staged copy of the colour after the last one is still in flight
    mbar_wait_bounded(&stage_bar, parity, exit_wait_limit(a.spin_limit), a.status);
    pending = false;
  }
  int info = 1;
  if (a.mode == 1) {
    // final full error (fc3d_nsgs.c:877-895)
    if (!full_error_phase(a, 5, epoch, full)) return;
    info = full < a.user_tol ? 0 : 1;
    if (sweep == a.max_sweeps && info > 0) info = -20;
  } else {
    info = converged ? 0 : 1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.out[0] = sweep;
    a.out[1] = incr;
    a.out[2] = full;
    a.out[3] = info;
    a.out[4] = working;
    a.out[5] = local_tol;
  }
}

}  // namespace fc3dgpu
