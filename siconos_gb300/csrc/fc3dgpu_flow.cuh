// Slab-dataflow FP32 sweep: the coloured Gauss-Seidel sweep without
// barriers between colours.
//
// The persistent sweep kernel (fc3dgpu_sweep.cuh) separates the colours of
// a sweep by block-level barriers, so every colour costs the slowest
// neighbour block's whole phase.  Here each warp owns whole 32-row slabs
// (slab s goes to warp s mod warps, so a warp meets its slabs in colour
// order).  Slab s must not start sweep k before, for every slab d holding
// a column of one of its rows (and every slab holding a row that reads one
// of s's columns: the neighbour lists are made symmetric),
//
//   d has updated its rows in sweep k      when d has an earlier colour,
//   d has updated its rows in sweep k - 1  when d has a later colour (its
//                     previous reactions, read before d may overwrite
//                     them: d waits for s),
//
// which is exactly the order of the sequential sweep in colour order
// (fc3d_nsgs.c:711-875 visiting the contacts colour by colour): every row
// reads the reactions a sequential sweep would read.
//
// Each slab carries an arrival counter that every neighbour increments
// after each of its updates.  A neighbour of an earlier colour cannot
// update sweep k + 1 before s has updated sweep k, and one of a later colour
// cannot update sweep k before s has, so while s waits for sweep k its
// counter never exceeds  n * k - n_later  (n neighbours, n_later of them of
// a later colour) and reaches it exactly when all of them are done: one
// acquire load of the slab's own counter replaces a load per neighbour.
// The (sweep, colour)
// order of the waits is acyclic and every warp is resident (cooperative
// launch), so the earliest unfinished slab can always proceed.  The light
// error of a sweep (fc3d_nsgs.c:80-96) and the stop rules still need one
// grid barrier per sweep.
//
// While a warp waits for a slab's columns, the bulk-copy engine brings that
// slab's W, column indices, q, diagonal block, mu and rho (one record per
// slab, packed before the sweeps) into the warp's shared-memory buffer; the
// next slab's copy is issued as soon as the current one's inputs are in
// registers.
#pragma once
#include "fc3dgpu_sweep.cuh"

namespace fc3dgpu {

// Polls of a slab's arrival counter before a warp starts to back off, and
// the back-off (ns) between later polls.
#define FC3D_FLOW_SPIN 1024
#define FC3D_FLOW_SLEEP_NS 64

// Stage slab s's record into the warp's buffer: one bulk copy completing
// on the warp's mbarrier (six copies from the separate arrays cost about
// 0.6 us of issue on the warp's chain of slabs).
// The record's place and size are loaded ahead (flow_next), so the issue
// does not wait for them on the warp's chain.
struct FlowNext {
  long long off;
  unsigned bytes;
};

__device__ __forceinline__ FlowNext flow_next(const SweepArgs<float>& a, const FlowArgs& f, int s) {
  FlowNext n;
  n.off = __ldg(&f.rec_off[s]);
  n.bytes = flow_rec_floats(__ldg(&a.slab_nslot[s])) * 4;
  return n;
}

__device__ __forceinline__ void flow_issue(const FlowArgs& f, const FlowNext& n, unsigned char* buf,
                                           unsigned long long* bar) {
  mbar_arrive_expect_tx(bar, n.bytes);
  bulk_g2s(buf, f.rec + n.off, n.bytes, bar);
}

// The per-slab records (flow_rec_floats) from the slab-major arrays of the
// layout; one block per slab at a time.  Run before a solve's FP32 sweeps
// (the arrays change with W, q and mu).
__global__ void k_flow_pack(int nslab, const long long* __restrict__ slab_off, const int* __restrict__ slab_nslot,
                            const float* __restrict__ W, const int* __restrict__ col, const float* __restrict__ q,
                            const float* __restrict__ D, const float* __restrict__ mu,
                            const float* __restrict__ rho, const long long* __restrict__ rec_off,
                            float* __restrict__ rec) {
  for (int s = blockIdx.x; s < nslab; s += gridDim.x) {
    const int ns = slab_nslot[s];
    const size_t o0 = (size_t)slab_off[s];
    float* R = rec + rec_off[s];
    const int nw = ns * 9 * FC3D_SLAB, ncl = ns * FC3D_SLAB;
    for (int i = threadIdx.x; i < nw; i += blockDim.x) R[i] = W[o0 * 9 * FC3D_SLAB + i];
    int* RC = reinterpret_cast<int*>(R + nw);
    for (int i = threadIdx.x; i < ncl; i += blockDim.x) RC[i] = col[o0 * FC3D_SLAB + i];
    float* RQ = R + nw + ncl;
    for (int i = threadIdx.x; i < 3 * FC3D_SLAB; i += blockDim.x) RQ[i] = q[(size_t)s * 3 * FC3D_SLAB + i];
    float* RD = RQ + 3 * FC3D_SLAB;
    for (int i = threadIdx.x; i < 9 * FC3D_SLAB; i += blockDim.x) RD[i] = D[(size_t)s * 9 * FC3D_SLAB + i];
    float* RM = RD + 9 * FC3D_SLAB;
    for (int i = threadIdx.x; i < FC3D_SLAB; i += blockDim.x) RM[i] = mu[(size_t)s * FC3D_SLAB + i];
    float* RR = RM + FC3D_SLAB;
    for (int i = threadIdx.x; i < 2 * FC3D_SLAB; i += blockDim.x) RR[i] = rho[(size_t)s * 2 * FC3D_SLAB + i];
  }
}

// Sum of N values over the block (fixed order), written to out_partials.
template <int N, int NW>
__device__ __forceinline__ void flow_block_sum(double v[N], double* out_partials) {
  __shared__ double sh[NW][8];
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
    for (int k = 0; k < NW; k++) s += sh[k][threadIdx.x];
    out_partials[threadIdx.x] = s;
  }
  __syncthreads();
}

template <int NW>
__device__ __forceinline__ bool flow_full_error(const SweepArgs<float>& a, unsigned& epoch, double& full) {
  double v[3];
  full_error_rows(a, v);
  flow_block_sum<3, NW>(v, a.partials + blockIdx.x * 8 + 2);
  if (!grid_barrier(a.barrier, epoch, a.spin_limit, a.status)) return false;
  double s[3];
  grid_sum<3>(a.partials, 2, s);
  double e = sqrt(s[0]);
  const double scal = fmax(a.norm_q, fmax(sqrt(s[2]), sqrt(s[1])));
  if (fabs(scal) > DBL_EPSILON) e /= scal;
  full = e;
  return true;
}

// Wait until every block's flag shows epoch e (bounded; warp 0 polls, then
// an acquire fence and a block barrier).  False when the wait gave up or a
// timeout anywhere is on record: one value for the whole block (read once,
// shared), so every warp leaves the sweep loop at the same barrier.
__device__ __forceinline__ bool grid_wait(const unsigned* flags, unsigned e, unsigned long long limit, int* status) {
  __shared__ int s_ok;
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    unsigned long long n = 0;
    int ok = 1;
    for (;;) {
      bool mine = true;
      for (int b = lane; b < (int)gridDim.x; b += 32)
        mine &= (ld_relaxed_u32(&flags[b * FC3D_FLAG_STRIDE]) >= e);
      if (__all_sync(0xffffffffu, mine)) break;
      if (++n > limit) {
        ok = 0;
        if (lane == 0) atomicOr(status, 1);
        break;
      }
      if (n > 256) __nanosleep(32);
    }
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    if (lane == 0) s_ok = ok && !(*(volatile int*)status & 1);
  }
  __syncthreads();
  return s_ok != 0;
}

// Wait until every neighbour slab of s has reached the state sweep k needs
// (see the header): one acquire load of s's arrival counter by every lane
// (one request for the warp) per poll.
__device__ __forceinline__ bool flow_wait_deps(const SweepArgs<float>& a, const FlowArgs& f, int s, unsigned target,
                                               int lane) {
  unsigned long long n = 0;
  bool ok = true;
  while (ld_acquire_u32(&f.done[s]) < target) {
    if (++n > a.spin_limit) {
      ok = false;
      if (lane == 0) atomicOr(a.status, 1);
      break;
    }
    if (n > FC3D_FLOW_SPIN) __nanosleep(FC3D_FLOW_SLEEP_NS);
  }
  return __all_sync(0xffffffffu, ok);
}

// Signal slab s's update to its neighbours: a fence orders the warp's
// reaction stores (made visible to this lane by the caller's __syncwarp)
// before the increments, which the waiting warps acquire.
// The lane's first two entries of the neighbour list come loaded (dep0,
// dep1), so no load waits between the fence and the increments for up to 64
// neighbours.
__device__ __forceinline__ void flow_signal(const FlowArgs& f, int d0, int d1, int dep0, int dep1, int lane) {
  __threadfence();
  const int i0 = d0 + lane;
  if (i0 < d1) atomicAdd(&f.done[dep0 & 0x7fffffff], 1u);
  if (i0 + 32 < d1) atomicAdd(&f.done[dep1 & 0x7fffffff], 1u);
  for (int i = i0 + 64; i < d1; i += 32) atomicAdd(&f.done[__ldg(&f.dep[i]) & 0x7fffffff], 1u);
}

// Row product, take-off test and local solve of the 32 rows of slab s from
// the warp's buffer; issues the copy of slab `next` (or none when next < 0)
// once the buffer is read.
// Inputs of slab s the columns' state does not affect: the row's presence,
// the slab's slot count, its neighbour list and wait rule (static, loaded a
// slab ahead by flow_static, so they are in registers when the slab starts)
// and the row's own reaction (only this warp writes it; loaded at the slab's
// start, with the wait for the column slabs).
struct FlowRow {
  bool row;
  int ns;
  float ro[3];
  int d0, d1, dep0, dep1;  // the slab's neighbour list, and this lane's first two entries
  unsigned need_a, need_b;  // wait for sweep k: counter >= need_a * k - need_b
};

__device__ __forceinline__ FlowRow flow_static(const SweepArgs<float>& a, const FlowArgs& f, int s, int lane) {
  FlowRow x;
  x.row = __ldg(&a.perm[s * FC3D_SLAB + lane]) >= 0;
  x.ns = __ldg(&a.slab_nslot[s]);
  x.d0 = __ldg(&f.dptr[s]);
  x.d1 = __ldg(&f.dptr[s + 1]);
  x.dep0 = x.d0 + lane < x.d1 ? __ldg(&f.dep[x.d0 + lane]) : 0;
  x.dep1 = x.d0 + lane + 32 < x.d1 ? __ldg(&f.dep[x.d0 + lane + 32]) : 0;
  const int2 nd = __ldg(&f.need[s]);
  x.need_a = (unsigned)nd.x;
  x.need_b = (unsigned)nd.y;
  x.ro[0] = x.ro[1] = x.ro[2] = 0.f;
  return x;
}

__device__ __forceinline__ void flow_own_r(const SweepArgs<float>& a, int s, int lane, FlowRow& x) {
  if (x.row) load_r3<float>(a.r, s * FC3D_SLAB + lane, x.ro);
}

// The new reaction of the lane's row goes to rn (zero on take-off); the
// light-error sums are left to the caller, after the slab's release.
__device__ __forceinline__ void flow_slab(const SweepArgs<float>& a, const FlowArgs& f, int s, const FlowNext& next,
                                          unsigned char* buf, unsigned long long* bar, int lane, float ltol,
                                          float rn[3], unsigned long long* tl, const FlowRow& x) {
  const int ns = x.ns;
  const float* Ws = reinterpret_cast<const float*>(buf);
  const int* Cs = reinterpret_cast<const int*>(buf + (size_t)ns * 9 * FC3D_SLAB * 4);
  const float* Qs = reinterpret_cast<const float*>(Cs + (size_t)ns * FC3D_SLAB);
  const float* Ds = Qs + 3 * FC3D_SLAB;
  const float* Ms = Ds + 9 * FC3D_SLAB;
  const float* Rs = Ms + FC3D_SLAB;
  const int p = s * FC3D_SLAB + lane;
  const float ro[3] = {x.ro[0], x.ro[1], x.ro[2]};
  float acc[3] = {0.f, 0.f, 0.f};
  bool work = false;
  LocalProblem<float> L;
  if (x.row) {
    acc[0] = Qs[lane];
    acc[1] = Qs[FC3D_SLAB + lane];
    acc[2] = Qs[2 * FC3D_SLAB + lane];
    constexpr int CH = 16;
    for (int t0 = 0; t0 < ns; t0 += CH) {
      float rv[CH][3];
#pragma unroll
      for (int k = 0; k < CH; k++) {
        const int pj = t0 + k < ns ? Cs[(t0 + k) * FC3D_SLAB + lane] : a.npad;
        load_r3<float>(a.r, pj, rv[k]);
      }
#pragma unroll
      for (int k = 0; k < CH; k++) {
        if (t0 + k < ns) {
          const float* wp = Ws + (size_t)(t0 + k) * 9 * FC3D_SLAB + lane;
          float wv[9];
#pragma unroll
          for (int e = 0; e < 9; e++) wv[e] = wp[e * FC3D_SLAB];
          mvp3x3(wv, rv[k], acc);
        }
      }
    }
    if (acc[0] > -Eps<float>::v()) {
      float* rp = a.r + (size_t)p * FC3D_RSTRIDE;
      rp[0] = 0;
      rp[1] = 0;
      rp[2] = 0;
    } else {
      work = true;
#pragma unroll
      for (int e = 0; e < 9; e++) L.M[e] = Ds[e * FC3D_SLAB + lane];
      L.mu = Ms[lane];
      L.rhoN = Rs[lane];
      L.rhoT = Rs[FC3D_SLAB + lane];
      L.q[0] = acc[0];
      L.q[1] = acc[1];
      L.q[2] = acc[2];
    }
  }
  const unsigned wmask = __ballot_sync(0xffffffffu, work);
  if (tl) {
    tl[3] = globaltimer_ns();
    tl[5] = (unsigned long long)__popc(wmask);
  }
  if (lane == 0) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    flow_issue(f, next, buf, bar);
  }
  if (tl) tl[6] = globaltimer_ns();
  rn[0] = rn[1] = rn[2] = 0.f;
  if (work) {
    L.rho_pli = __ldcg(&a.rpli[p]);
    L.tol = ltol;
    L.newton_max = a.newton_max;
    L.pli_max = a.pli_max;
    L.ls_max = a.ls_max;
    L.mode = a.local_mode;
    L.n_newton = L.n_pli = L.n_ls = 0;
    rn[0] = ro[0];
    rn[1] = ro[1];
    rn[2] = ro[2];
    local_solve(L, rn);
    float* rp = a.r + (size_t)p * FC3D_RSTRIDE;
    rp[0] = rn[0];
    rp[1] = rn[1];
    rp[2] = rn[2];
    a.rpli[p] = L.rho_pli;
  }
  __syncwarp();
  if (tl) tl[7] = globaltimer_ns();
}

template <int NW>
__global__ void __launch_bounds__(NW * 32, 1) nsgs_flow_kernel(const SweepArgs<float> a, const FlowArgs f) {
  extern __shared__ __align__(128) unsigned char flow_smem[];
  __shared__ __align__(8) unsigned long long bars[NW];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* buf = flow_smem + (size_t)w * f.buf_bytes;
  unsigned long long* bar = &bars[w];
  if (lane == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  const int gw = blockIdx.x * NW + w, tw = gridDim.x * NW;
  unsigned parity = 0;
  bool pending = false, failed = false;
  FlowRow xs;  // the static inputs of the warp's next slab
  if (gw < a.nslab) {
    if (lane == 0) flow_issue(f, flow_next(a, f, gw), buf, bar);
    pending = true;
    xs = flow_static(a, f, gw, lane);
  }
  // Light errors run one sweep behind: at the end of sweep j a block
  // publishes its partial sums of sweep j (slot j mod 4 of f.part) and its
  // arrival, then waits only for every block's arrival at the end of sweep
  // j - 1 (long past, as a rule) and decides on sweep j - 1's light error:
  // no grid barrier between sweeps.  A stop so decided takes effect after
  // sweep j.  Four slots: when a block writes slot j mod 4, every block has
  // read it (at the end of sweep j - 3; the block saw all arrivals of the
  // end of sweep j - 2).  The full error needs one iterate everywhere, so it
  // waits for every block's end of sweep j.
  unsigned epoch = 0, e_last = 0, e_prev = 0;
  double working = fmax(a.user_tol, a.switch_tol);
  double incr = INFINITY, full = INFINITY, best = INFINITY;
  int sweep = 0, best_sweep = 0;
  bool converged = false, aborted = false, stopped = false;
  const double target = fmax(a.user_tol, a.switch_tol);
  auto light_error = [&](int j) {
    double sm[2];
    grid_sum<2>(f.part, (j & 3) * 2, sm);
    double e = sqrt(sm[0]);
    const double nr = sqrt(sm[1]);
    if (fabs(nr) > DBL_EPSILON) e /= nr;
    if (a.trace && blockIdx.x == 0 && threadIdx.x == 0 && a.trace_base + j - 1 < a.trace_cap)
      a.trace[a.trace_base + j - 1] = e;
    return e;
  };
  // the full error of the current iterate once every block ended sweep j
  // (epoch e_end); adapts the working tolerance as the coloured kernel does
  auto full_check = [&](double incr_j, unsigned e_end) {
    if (!grid_wait(a.barrier, e_end, a.spin_limit, a.status)) return false;
    if (!flow_full_error<NW>(a, epoch, full)) return false;
    if (full <= target) {
      converged = true;
    } else if (full > 0.0 && incr_j > 0.0) {
      double nt = (incr_j / full) * target;
      const double mint = fmax(target * 1e-6, DBL_EPSILON * 1e-6);
      if (nt < mint) nt = mint;
      if (nt < working) working = nt;
    }
    return true;
  };
  while (sweep < a.max_sweeps) {
    sweep++;
    double acc[2] = {0.0, 0.0};
    const bool record = a.timeline && sweep == a.timeline_sweep && lane == 0;
    for (int s = gw; s < a.nslab && !failed; s += tw) {
      unsigned long long* tl = record ? a.timeline + (size_t)s * FC3D_TL_STRIDE : nullptr;
      if (tl) tl[0] = globaltimer_ns();
      // the next slab of this warp: later in this sweep, else the first one
      // of the next sweep (fetched even when no sweep follows; awaited at exit)
      const int sn = s + tw < a.nslab ? s + tw : gw;
      const FlowNext next = flow_next(a, f, sn);
      FlowRow x = xs;
      xs = flow_static(a, f, sn, lane);
      flow_own_r(a, s, lane, x);
      if (!flow_wait_deps(a, f, s, x.need_a * (unsigned)sweep - x.need_b, lane)) {
        failed = true;
        break;
      }
      __syncwarp();
      if (tl) tl[1] = globaltimer_ns();
      if (pending) {
        if (!mbar_wait_bounded(bar, parity, a.spin_limit, a.status)) {
          failed = true;  // the copy stays pending: awaited again at exit
          break;
        }
        parity ^= 1u;
        pending = false;
      }
      if (tl) tl[2] = globaltimer_ns();
      float rn[3];
      flow_slab(a, f, s, next, buf, bar, lane, (float)a.local_tol, rn, tl, x);
      pending = true;
      if (x.row) {
        // light-error sums (fc3d_nsgs.c:80-96), while the reaction stores
        // drain: squares in FP32, sums in FP64 (the FP64 pipe is a small
        // share of the SM's)
        const float d0 = x.ro[0] - rn[0], d1 = x.ro[1] - rn[1], d2 = x.ro[2] - rn[2];
        acc[0] += (double)(d0 * d0 + d1 * d1 + d2 * d2);
        acc[1] += (double)(rn[0] * rn[0] + rn[1] * rn[1] + rn[2] * rn[2]);
      }
      __syncwarp();
      if (tl) tl[4] = globaltimer_ns();
      flow_signal(f, x.d0, x.d1, x.dep0, x.dep1, lane);
    }
    flow_block_sum<2, NW>(acc, f.part + blockIdx.x * 8 + (sweep & 3) * 2);
    e_prev = e_last;
    e_last = ++epoch;
    if (threadIdx.x == 0) st_release_u32(&a.barrier[blockIdx.x * FC3D_FLAG_STRIDE], e_last);
    if (sweep < 2) continue;
    if (!grid_wait(a.barrier, e_prev, a.spin_limit, a.status)) {
      aborted = true;
      break;
    }
    // the FP32 accelerator's stop rules on sweep - 1, as the coloured
    // kernel applies them to each sweep
    const double e1 = light_error(sweep - 1);
    bool stop = false;
    if (!(e1 == e1)) {
      if (threadIdx.x == 0) atomicOr(a.status, 2);
      stop = true;
    }
    if (e1 < a.switch_tol) stop = true;
    if (e1 < 0.99 * best) {
      best = e1;
      best_sweep = sweep - 1;
    } else if (a.stall_window > 0 && sweep - 1 - best_sweep >= a.stall_window) {
      stop = true;
    }
    if (!stop && e1 < working) {
      if (!full_check(e1, e_last)) {
        aborted = true;
        break;
      }
      stop = converged;
    }
    if (stop) {
      stopped = true;
      break;
    }
  }
  if (sweep > 0 && !aborted) {
    // the light error of the last sweep; after a budget end, the stop rules
    // on it as on every other sweep
    if (!grid_wait(a.barrier, e_last, a.spin_limit, a.status)) {
      aborted = true;
    } else {
      incr = light_error(sweep);
      if (!stopped) {
        bool stop = false;
        if (!(incr == incr)) {
          if (threadIdx.x == 0) atomicOr(a.status, 2);
          stop = true;
        }
        if (incr < a.switch_tol) stop = true;
        if (!stop && incr < working) aborted = !full_check(incr, e_last);
      }
    }
  }
  // a copy still in flight lands before the block leaves
  if (pending) mbar_wait_bounded(bar, parity, exit_wait_limit(a.spin_limit), a.status);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.out[0] = sweep;
    a.out[1] = incr;
    a.out[2] = full;
    a.out[3] = converged ? 0 : 1;
    a.out[4] = working;
    a.out[5] = a.local_tol;
  }
}

// Column slabs of every slab: the distinct slabs holding a column of one of
// its rows.  One thread per slab; with dptr null it writes their number to
// count[s], else the ascending list to dep[dptr[s] ..), bit 31 set for a
// later colour.  Slabs have at most FC3D_FLOW_MAXSLOT slots.
__global__ void k_flow_deps(int nslab, int npad, int ncol, const int* __restrict__ sptr_d,
                            const int* __restrict__ perm, const int* __restrict__ slab_nslot,
                            const long long* __restrict__ slab_off, const int* __restrict__ col,
                            const int* __restrict__ dptr, int* __restrict__ count, int* __restrict__ dep) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslab) return;
  auto colour_of = [&](int sl) {
    int lo = 0, hi = ncol - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sptr_d[mid] <= sl)
        lo = mid;
      else
        hi = mid - 1;
    }
    return lo;
  };
  int list[FC3D_SLAB * FC3D_FLOW_MAXSLOT];
  int n = 0;
  const int ns = min(slab_nslot[s], FC3D_FLOW_MAXSLOT);
  const long long base = slab_off[s];
  for (int k = 0; k < FC3D_SLAB; k++) {
    if (perm[(size_t)s * FC3D_SLAB + k] < 0) continue;
    for (int t = 0; t < ns; t++) {
      const int j = col[(size_t)(base + t) * FC3D_SLAB + k];
      if (j < 0 || j >= npad) continue;
      const int d = j / FC3D_SLAB;
      bool seen = d == s;
      for (int i = 0; i < n && !seen; i++) seen = list[i] == d;
      if (!seen) list[n++] = d;
    }
  }
  if (!dptr) {
    count[s] = n;
    return;
  }
  for (int i = 1; i < n; i++) {
    const int v = list[i];
    int j = i - 1;
    while (j >= 0 && list[j] > v) {
      list[j + 1] = list[j];
      j--;
    }
    list[j + 1] = v;
  }
  const int cs = colour_of(s);
  int* out = dep + dptr[s];
  for (int i = 0; i < n; i++) out[i] = colour_of(list[i]) > cs ? (int)(list[i] | 0x80000000u) : list[i];
}

}  // namespace fc3dgpu
