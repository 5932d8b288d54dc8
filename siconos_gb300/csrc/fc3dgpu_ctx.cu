// Device-side set-up of a problem: Jones-Plassmann colouring of the contact
// conflict graph, stable permutation of the rows by colour into 32-row slabs,
// and the slot-major block layout (fc3dgpu_layout.cuh).  Everything here runs
// once per W; the sweeps never touch the block-CSR input again.
//
// Colouring.  The reference colours the conflict graph with PETSc's greedy
// distance-1 colouring (tools/parallel/graph_tools.c:876-928).  Here every
// contact gets a 32-bit priority (an integer hash of its index, optionally
// led by its conflict degree); a contact is coloured once all its
// higher-priority neighbours are, with the smallest colour none of them
// holds.  That equals sequential greedy colouring in decreasing priority, so
// the result is deterministic and matches the host greedy colouring of the
// same graph.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fc3dgpu_batch_args.cuh"
#include "fc3dgpu_sweep_launch.h"
#include "fc3dgpu_fast64.h"
#include "fc3dgpu_layout.cuh"
#include "fc3dgpu_local.cuh"
#include "fc3dgpu_mlp.h"

namespace fc3dgpu {

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
  // lowbias32 (C. Wellons)
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ uint32_t colour_priority(uint32_t index, int kind, uint32_t degree) {
  uint32_t h = hash32(index ^ 0x9e3779b9U);
  if (kind == 1) return ((degree > 255 ? 255U : degree) << 24) | (h >> 8);
  return h;
}

__global__ void k_degree(int nc, const long long* __restrict__ rowptr, const long long* __restrict__ colidx,
                         int* __restrict__ deg) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x)
    for (long long k = rowptr[i]; k < rowptr[i + 1]; k++) {
      long long j = colidx[k];
      if (j == i) continue;
      atomicAdd(&deg[i], 1);
      atomicAdd(&deg[j], 1);
    }
}

__global__ void k_adjacency(int nc, const long long* __restrict__ rowptr, const long long* __restrict__ colidx,
                            int* __restrict__ cursor, int* __restrict__ adj) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x)
    for (long long k = rowptr[i]; k < rowptr[i + 1]; k++) {
      long long j = colidx[k];
      if (j == i) continue;
      adj[atomicAdd(&cursor[i], 1)] = (int)j;
      adj[atomicAdd(&cursor[j], 1)] = i;
    }
}

// priority keys; kind 1 counts distinct neighbours (a pair may appear as
// both (i,j) and (j,i) in W)
__global__ void k_priority(int nc, const int* __restrict__ gptr, const int* __restrict__ adj, int kind,
                           uint32_t* __restrict__ key, int* __restrict__ colour, const int* __restrict__ grp,
                           const int* __restrict__ group_off) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
    uint32_t d = 0;
    if (kind == 1)
      for (int k = gptr[i]; k < gptr[i + 1]; k++) {
        bool dup = false;
        for (int m = gptr[i]; m < k; m++)
          if (adj[m] == adj[k]) {
            dup = true;
            break;
          }
        d += dup ? 0 : 1;
      }
    // batched problems: the index inside the problem, so each problem is
    // coloured exactly as it would be alone
    const int local = grp ? i - group_off[grp[i]] : i;
    key[i] = colour_priority((uint32_t)local, kind, d);
    colour[i] = -1;
  }
}

// Iterated greedy (Culberson): recolour with the current colour classes
// visited as blocks in reverse order (highest colour first; hash inside a
// class).  Members of a class are independent, so greedy over whole classes
// never needs more colours than there are classes, and the small last
// classes tend to dissolve into the others.
__global__ void k_recolour_key(int nc, const int* __restrict__ grp, const int* __restrict__ group_off,
                               uint32_t* __restrict__ key, int* __restrict__ colour) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
    const int local = grp ? i - group_off[grp[i]] : i;
    key[i] = ((uint32_t)colour[i] << 24) | (colour_priority((uint32_t)local, 0, 0) >> 8);
    colour[i] = -1;
  }
}

__global__ void k_jp_round(int nc, const int* __restrict__ gptr, const int* __restrict__ adj,
                           const uint32_t* __restrict__ key, int* colour, int* remaining, int* overflow) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
    if (((volatile int*)colour)[i] >= 0) continue;
    const uint32_t ki = key[i];
    unsigned long long used0 = 0, used1 = 0;
    bool ready = true;
    for (int k = gptr[i]; k < gptr[i + 1]; k++) {
      const int w = adj[k];
      const uint32_t kw = key[w];
      if (!(kw > ki || (kw == ki && w < i))) continue;  // lower priority
      const int c = ((volatile int*)colour)[w];
      if (c < 0) {
        ready = false;
        break;
      }
      if (c < 64)
        used0 |= 1ULL << c;
      else if (c < 128)
        used1 |= 1ULL << (c - 64);
    }
    if (!ready) {
      atomicAdd(remaining, 1);
      continue;
    }
    int c = __ffsll(~used0) - 1;
    if (c < 0 || used0 == ~0ULL) {
      int c1 = __ffsll(~used1) - 1;
      c = (c1 < 0) ? 128 : 64 + c1;
    }
    if (c >= FC3D_MAX_COLOURS) {
      atomicOr(overflow, 1);
      c = FC3D_MAX_COLOURS - 1;
    }
    ((volatile int*)colour)[i] = c;
  }
}

// per 1024-contact block: colour histogram
__global__ void k_colour_hist(int nc, const int* __restrict__ colour, int* __restrict__ blockhist) {
  __shared__ int h[FC3D_MAX_COLOURS];
  for (int c = threadIdx.x; c < FC3D_MAX_COLOURS; c += blockDim.x) h[c] = 0;
  __syncthreads();
  const int i = blockIdx.x * 1024 + threadIdx.x;
  if (i < nc) atomicAdd(&h[colour[i]], 1);
  __syncthreads();
  for (int c = threadIdx.x; c < FC3D_MAX_COLOURS; c += blockDim.x) blockhist[blockIdx.x * FC3D_MAX_COLOURS + c] = h[c];
}

// single block: per-(colour, block) offsets inside each colour, colour
// counts and slab ranges
__global__ void k_colour_offsets(int nblocks, int* __restrict__ blockhist, int* __restrict__ counts,
                                 int* __restrict__ sptr) {
  const int c = threadIdx.x;
  if (c < FC3D_MAX_COLOURS) {
    int run = 0;
    for (int b = 0; b < nblocks; b++) {
      int v = blockhist[b * FC3D_MAX_COLOURS + c];
      blockhist[b * FC3D_MAX_COLOURS + c] = run;
      run += v;
    }
    counts[c] = run;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    sptr[0] = 0;
    for (int k = 0; k < FC3D_MAX_COLOURS; k++) {
      s += (counts[k] + FC3D_SLAB - 1) / FC3D_SLAB;
      sptr[k + 1] = s;
    }
  }
}

// stable scatter: contacts keep index order inside their colour
__global__ void k_colour_scatter(int nc, const int* __restrict__ colour, const int* __restrict__ blockoff,
                                 const int* __restrict__ sptr, int* __restrict__ perm, int* __restrict__ iperm) {
  __shared__ int wcount[32][FC3D_MAX_COLOURS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int t = threadIdx.x; t < 32 * FC3D_MAX_COLOURS; t += blockDim.x) (&wcount[0][0])[t] = 0;
  __syncthreads();
  const int i = blockIdx.x * 1024 + threadIdx.x;
  const int c = (i < nc) ? colour[i] : -1;
  const unsigned mask = __match_any_sync(0xffffffffu, c);
  const int leader = __ffs(mask) - 1;
  if (c >= 0 && lane == leader) wcount[w][c] = __popc(mask);
  __syncthreads();
  // exclusive prefix over warps, per colour
  for (int cc = threadIdx.x; cc < FC3D_MAX_COLOURS; cc += blockDim.x) {
    int run = 0;
    for (int k = 0; k < 32; k++) {
      int v = wcount[k][cc];
      wcount[k][cc] = run;
      run += v;
    }
  }
  __syncthreads();
  if (c >= 0) {
    const int rank = blockoff[blockIdx.x * FC3D_MAX_COLOURS + c] + wcount[w][c] + __popc(mask & ((1u << lane) - 1));
    const int p = sptr[c] * FC3D_SLAB + rank;
    perm[p] = i;
    iperm[i] = p;
  }
}

// per padded row: off-diagonal count and slot position of the diagonal
__global__ void k_rowinfo(int npad, const int* __restrict__ perm, const long long* __restrict__ rowptr,
                          const long long* __restrict__ colidx, int* __restrict__ rowlen, int* __restrict__ dpos,
                          int* __restrict__ nodiag) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npad; p += gridDim.x * blockDim.x) {
    const int i = perm[p];
    if (i < 0) {
      rowlen[p] = 0;
      dpos[p] = 0;
      continue;
    }
    int s = 0, d = -1;
    for (long long k = rowptr[i]; k < rowptr[i + 1]; k++) {
      if (colidx[k] == i && d < 0)
        d = s;
      else
        s++;
    }
    rowlen[p] = s;
    dpos[p] = d < 0 ? s : d;
    if (d < 0) atomicOr(nodiag, 1);
  }
}

__global__ void k_slab_nslot(int nslab, const int* __restrict__ rowlen, int* __restrict__ nslot) {
  const int lane = threadIdx.x & 31;
  const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (s >= nslab) return;
  int v = rowlen[s * FC3D_SLAB + lane];
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (lane == 0) nslot[s] = v;
}

// single block: exclusive scan (64-bit output) of n counts; total in *total
template <typename In>
__global__ void k_scan_excl(int n, const In* __restrict__ cnt, long long* __restrict__ off, long long* __restrict__ total) {
  __shared__ long long carry;
  __shared__ long long buf[1024];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int t = threadIdx.x, idx = base + t;
    buf[t] = idx < n ? (long long)cnt[idx] : 0;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      long long v = t >= o ? buf[t - o] : 0;
      __syncthreads();
      buf[t] += v;
      __syncthreads();
    }
    if (idx < n) off[idx] = carry + buf[t] - (long long)cnt[idx];
    __syncthreads();
    if (t == 1023) carry += buf[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void k_ll_to_int(int n, const long long* __restrict__ a, int* __restrict__ b) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) b[t] = (int)a[t];
}

__global__ void k_max_colour(int nc, const int* __restrict__ colour, int* __restrict__ mx) {
  int m = -1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) m = max(m, colour[i]);
  for (int o = 16; o >= 1; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
}

__global__ void k_fill_col_pad(long long nslots, int npad, int* __restrict__ col) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nslots * FC3D_SLAB;
       t += (long long)gridDim.x * blockDim.x)
    col[t] = npad;
}

// scatter the blocks of each row into the slab layout (FP64 master copy)
// One thread per padded row, in slab order: the 32 rows of a slab write
// each slot's element e as one coalesced line.
__global__ void k_fill_blocks(int npad, const int* __restrict__ perm, const long long* __restrict__ rowptr,
                              const long long* __restrict__ colidx, const double* __restrict__ blocks,
                              const int* __restrict__ iperm, const long long* __restrict__ slab_off,
                              double* __restrict__ W, int* __restrict__ col, double* __restrict__ D,
                              double* __restrict__ rho) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npad; p += gridDim.x * blockDim.x) {
    const int i = perm[p];
    if (i < 0) continue;
    const int slab = p / FC3D_SLAB, k = p % FC3D_SLAB;
    const long long base = slab_off[slab];
    int s = 0;
    bool diag_done = false;
    for (long long kk = rowptr[i]; kk < rowptr[i + 1]; kk++) {
      const long long j = colidx[kk];
      const double* b = blocks + 9 * kk;
      if (j == i && !diag_done) {
        diag_done = true;
        for (int e = 0; e < 9; e++) D[((size_t)slab * 9 + e) * FC3D_SLAB + k] = b[e];
      } else {
        const size_t sl = (size_t)(base + s);
        for (int e = 0; e < 9; e++) W[(sl * 9 + e) * FC3D_SLAB + k] = b[e];
        col[sl * FC3D_SLAB + k] = iperm[j];
        s++;
      }
    }
    double M[9];
    for (int e = 0; e < 9; e++) M[e] = D[((size_t)slab * 9 + e) * FC3D_SLAB + k];
    double rn = 1.0, rt = 1.0;
    if (diag_done) ac_rho<double>(M, rn, rt);
    rho[((size_t)slab * 2) * FC3D_SLAB + k] = rn;
    rho[((size_t)slab * 2 + 1) * FC3D_SLAB + k] = rt;
  }
}

__global__ void k_to_f32(long long n, const double* __restrict__ a, float* __restrict__ b) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    b[t] = (float)a[t];
}

__global__ void k_set_q_mu(int nc, const int* __restrict__ iperm, const double* __restrict__ q,
                           const double* __restrict__ mu, double* __restrict__ q64, double* __restrict__ mu64,
                           float* __restrict__ q32, float* __restrict__ mu32) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
    const int p = iperm[i], slab = p / FC3D_SLAB, k = p % FC3D_SLAB;
    for (int a = 0; a < 3; a++) {
      const double v = q[3 * (size_t)i + a];
      q64[((size_t)slab * 3 + a) * FC3D_SLAB + k] = v;
      q32[((size_t)slab * 3 + a) * FC3D_SLAB + k] = (float)v;
    }
    mu64[(size_t)slab * FC3D_SLAB + k] = mu[i];
    mu32[(size_t)slab * FC3D_SLAB + k] = (float)mu[i];
  }
}

// ---- batched problems: per-problem permutation by colour ----------------

__global__ void k_group_ids(int ngroups, const int* __restrict__ group_off, int* __restrict__ grp) {
  const int g = blockIdx.x;
  if (g >= ngroups) return;
  for (int i = group_off[g] + threadIdx.x; i < group_off[g + 1]; i += blockDim.x) grp[i] = g;
}

// one block per problem: colour counts, colours used, slabs needed
__global__ void k_scene_counts(const int* __restrict__ group_off, const int* __restrict__ colour,
                               int* __restrict__ scounts, int* __restrict__ snslab, int* __restrict__ sncol) {
  __shared__ int h[FC3D_MAX_COLOURS];
  const int g = blockIdx.x;
  for (int k = threadIdx.x; k < FC3D_MAX_COLOURS; k += blockDim.x) h[k] = 0;
  __syncthreads();
  for (int i = group_off[g] + threadIdx.x; i < group_off[g + 1]; i += blockDim.x) atomicAdd(&h[colour[i]], 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    int ns = 0, nc = 0;
    for (int k = 0; k < FC3D_MAX_COLOURS; k++) {
      scounts[(size_t)g * FC3D_MAX_COLOURS + k] = h[k];
      ns += (h[k] + FC3D_SLAB - 1) / FC3D_SLAB;
      if (h[k]) nc = k + 1;
    }
    snslab[g] = ns;
    sncol[g] = nc;
  }
}

// one block per problem: slab table and stable scatter (index order kept
// inside each colour), chunk by chunk with a running count per colour
__global__ void k_scene_scatter(const int* __restrict__ group_off, const int* __restrict__ colour,
                                const int* __restrict__ scounts, const long long* __restrict__ sbase,
                                int* __restrict__ ssptr, int* __restrict__ perm, int* __restrict__ iperm) {
  __shared__ int sptr[FC3D_MAX_COLOURS + 1];
  __shared__ int carry[FC3D_MAX_COLOURS];
  __shared__ int chunk_tot[FC3D_MAX_COLOURS];
  __shared__ int wcount[32][FC3D_MAX_COLOURS];
  const int g = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    int sl = (int)sbase[g];
    sptr[0] = sl;
    for (int k = 0; k < FC3D_MAX_COLOURS; k++) {
      sl += (scounts[(size_t)g * FC3D_MAX_COLOURS + k] + FC3D_SLAB - 1) / FC3D_SLAB;
      sptr[k + 1] = sl;
    }
  }
  for (int k = threadIdx.x; k < FC3D_MAX_COLOURS; k += blockDim.x) carry[k] = 0;
  __syncthreads();
  for (int k = threadIdx.x; k <= FC3D_MAX_COLOURS; k += blockDim.x)
    ssptr[(size_t)g * (FC3D_MAX_COLOURS + 1) + k] = sptr[k];
  for (int base = group_off[g]; base < group_off[g + 1]; base += blockDim.x) {
    for (int t = threadIdx.x; t < 32 * FC3D_MAX_COLOURS; t += blockDim.x) (&wcount[0][0])[t] = 0;
    __syncthreads();
    const int i = base + threadIdx.x;
    const int c = i < group_off[g + 1] ? colour[i] : -1;
    const unsigned mask = __match_any_sync(0xffffffffu, c);
    if (c >= 0 && lane == __ffs(mask) - 1) wcount[w][c] = __popc(mask);
    __syncthreads();
    // exclusive prefix over warps per colour; chunk totals kept aside
    for (int cc = threadIdx.x; cc < FC3D_MAX_COLOURS; cc += blockDim.x) {
      int run = 0;
      for (int k = 0; k < 32; k++) {
        const int v = wcount[k][cc];
        wcount[k][cc] = run;
        run += v;
      }
      chunk_tot[cc] = run;
    }
    __syncthreads();
    if (c >= 0) {
      const int rank = carry[c] + wcount[w][c] + __popc(mask & ((1u << lane) - 1));
      const int p = sptr[c] * FC3D_SLAB + rank;
      perm[p] = i;
      iperm[i] = p;
    }
    __syncthreads();
    for (int cc = threadIdx.x; cc < FC3D_MAX_COLOURS; cc += blockDim.x) carry[cc] += chunk_tot[cc];
    __syncthreads();
  }
}

// per-problem FP64 budget after the FP32 phase
__global__ void k_batch_budget(int n, const double* __restrict__ out32, int max_iter, int* __restrict__ budget) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const int b = max_iter - (int)out32[(size_t)s * 8];
    budget[s] = b > 0 ? b : 0;
  }
}

// r (original order, 3 per contact) -> padded AoS copies; PLI step reset to 1
// as fc3d_AC_initialize does at every solve (onecontact.c:115)
__global__ void k_set_r(int nc, const int* __restrict__ iperm, const double* __restrict__ r, double* __restrict__ r64,
                        float* __restrict__ r32, double* __restrict__ rpli64, float* __restrict__ rpli32) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
    const int p = iperm[i];
    for (int a = 0; a < 3; a++) {
      r64[4 * (size_t)p + a] = r[3 * (size_t)i + a];
      r32[4 * (size_t)p + a] = (float)r[3 * (size_t)i + a];
    }
    rpli64[p] = 1.0;
    rpli32[p] = 1.0f;
  }
}

__global__ void k_r32_to_r64(int npad, const float* __restrict__ r32, const float* __restrict__ rpli32,
                             double* __restrict__ r64, double* __restrict__ rpli64) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npad; p += gridDim.x * blockDim.x) {
    for (int a = 0; a < 3; a++) r64[4 * (size_t)p + a] = (double)r32[4 * (size_t)p + a];
    rpli64[p] = (double)rpli32[p];
  }
}

__global__ void k_r64_to_r32(int npad, const double* __restrict__ r64, float* __restrict__ r32) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npad; p += gridDim.x * blockDim.x)
    for (int a = 0; a < 3; a++) r32[4 * (size_t)p + a] = (float)r64[4 * (size_t)p + a];
}

// The 17 warm-start features of every row (padding rows: zeros): the
// diagonal block (column-major), q, mu, the current reaction, the gap of
// the row's contact (gapo in the caller's order, or 0).
__global__ void k_features(int npad, const int* __restrict__ perm, const double* __restrict__ D64,
                           const double* __restrict__ q64, const double* __restrict__ mu64,
                           const double* __restrict__ r64, const double* __restrict__ gapo, float* __restrict__ X) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npad; p += gridDim.x * blockDim.x) {
    float* x = X + (size_t)p * FC3DGPU_MLP_FEATURES;
    const int i = perm[p];
    if (i < 0) {
      for (int f = 0; f < FC3DGPU_MLP_FEATURES; f++) x[f] = 0.f;
      continue;
    }
    const int slab = p / FC3D_SLAB, k = p % FC3D_SLAB;
    for (int e = 0; e < 9; e++) x[e] = (float)D64[((size_t)slab * 9 + e) * FC3D_SLAB + k];
    for (int a = 0; a < 3; a++) x[9 + a] = (float)q64[(size_t)slab * 3 * FC3D_SLAB + a * FC3D_SLAB + k];
    x[12] = (float)mu64[(size_t)slab * FC3D_SLAB + k];
    for (int a = 0; a < 3; a++) x[13 + a] = (float)r64[4 * (size_t)p + a];
    x[16] = gapo ? (float)gapo[i] : 0.f;
  }
}

__global__ void k_gather_features(int nc, const int* __restrict__ iperm, const float* __restrict__ Xp,
                                  float* __restrict__ X) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)nc * FC3DGPU_MLP_FEATURES;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / FC3DGPU_MLP_FEATURES), f = (int)(e % FC3DGPU_MLP_FEATURES);
    X[e] = Xp[(size_t)iperm[i] * FC3DGPU_MLP_FEATURES + f];
  }
}

// The candidate prev + alpha (target - prev), projected on each row's
// friction cone, in place of the current reaction; prev is the reaction
// before the warm start, saved in rbak on the first candidate (save != 0).
// target is the network's output Y, or prev + Y for a network that predicts
// the change of the reaction (residual != 0).
__global__ void k_take_proposal(int npad, const int* __restrict__ perm, const float* __restrict__ Y,
                                const double* __restrict__ mu64, double* __restrict__ r64, float* __restrict__ r32,
                                double* __restrict__ rbak, double alpha, int residual, int save) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npad; p += gridDim.x * blockDim.x) {
    if (save)
      for (int a = 0; a < 3; a++) rbak[4 * (size_t)p + a] = r64[4 * (size_t)p + a];
    if (perm[p] < 0) continue;
    double r[3];
    for (int a = 0; a < 3; a++) {
      const double prev = rbak[4 * (size_t)p + a], y = (double)Y[3 * (size_t)p + a];
      const double target = residual ? prev + y : y;
      r[a] = prev + alpha * (target - prev);
    }
    const int slab = p / FC3D_SLAB, k = p % FC3D_SLAB;
    project_cone<double>(r, mu64[(size_t)slab * FC3D_SLAB + k]);
    for (int a = 0; a < 3; a++) {
      r64[4 * (size_t)p + a] = r[a];
      r32[4 * (size_t)p + a] = (float)r[a];
    }
  }
}

struct ColourBounds {
  int sptr[FC3D_MAX_COLOURS + 1];
};

// Block that processes slab s in a sweep over `grid` blocks: the colour's
// slabs are split as block_range does, [s0 + n b / grid, s0 + n (b+1) / grid).
__device__ __forceinline__ int owner_block(int s, const ColourBounds& cb, int ncol, int grid) {
  int lo = 0, hi = ncol - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (cb.sptr[mid] <= s)
      lo = mid;
    else
      hi = mid - 1;
  }
  const int s0 = cb.sptr[lo], n = cb.sptr[lo + 1] - s0, x = s - s0;
  int b = (int)(((long long)x * grid) / n);
  if (b >= grid) b = grid - 1;
  while (b + 1 < grid && (long long)n * (b + 1) / grid <= x) b++;
  while (b > 0 && (long long)n * b / grid > x) b--;
  return b;
}

// mask[b][b' / 32] bit b' % 32 set when a row of block b and a row of block
// b' share a W block (both directions).
__global__ void k_block_adjacency(int nslab, int npad, ColourBounds cb, int ncol, int grid, int words,
                                  const int* __restrict__ perm, const int* __restrict__ slab_nslot,
                                  const long long* __restrict__ slab_off, const int* __restrict__ col,
                                  unsigned* __restrict__ mask) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)nslab * FC3D_SLAB;
       t += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(t / FC3D_SLAB), k = (int)(t % FC3D_SLAB);
    if (perm[(size_t)s * FC3D_SLAB + k] < 0) continue;
    const int b = owner_block(s, cb, ncol, grid);
    const int ns = slab_nslot[s];
    const long long base = slab_off[s];
    for (int slot = 0; slot < ns; slot++) {
      const int j = col[(size_t)(base + slot) * FC3D_SLAB + k];
      if (j < 0 || j >= npad) continue;
      const int bj = owner_block(j / FC3D_SLAB, cb, ncol, grid);
      if (bj == b) continue;
      unsigned* m1 = &mask[(size_t)b * words + bj / 32];
      unsigned* m2 = &mask[(size_t)bj * words + b / 32];
      if (!(*(volatile unsigned*)m1 & (1u << (bj % 32)))) atomicOr(m1, 1u << (bj % 32));
      if (!(*(volatile unsigned*)m2 & (1u << (b % 32)))) atomicOr(m2, 1u << (b % 32));
    }
  }
}

__global__ void k_restore_r(int npad, const double* __restrict__ rbak, double* __restrict__ r64,
                            float* __restrict__ r32) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npad; p += gridDim.x * blockDim.x)
    for (int a = 0; a < 3; a++) {
      r64[4 * (size_t)p + a] = rbak[4 * (size_t)p + a];
      r32[4 * (size_t)p + a] = (float)rbak[4 * (size_t)p + a];
    }
}

__global__ void k_get_r_u(int nc, const int* __restrict__ iperm, const double* __restrict__ r64,
                          const double* __restrict__ u64, double* __restrict__ r, double* __restrict__ u) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
    const int p = iperm[i];
    for (int a = 0; a < 3; a++) {
      if (r) r[3 * (size_t)i + a] = r64[4 * (size_t)p + a];
      if (u) u[3 * (size_t)i + a] = u64[3 * (size_t)p + a];
    }
  }
}

}  // namespace fc3dgpu

// ---------------------------------------------------------------------------
// Device context (C-ABI in include/fc3dgpu.h)
// ---------------------------------------------------------------------------
#include <math.h>
#include <stdarg.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <memory>
#include <thread>
#include <vector>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fc3dgpu.h"

static thread_local char g_err[512];

extern "C" const char* fc3dgpu_last_error(void) { return g_err; }

extern "C" void fc3dgpu_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

#define CK(x)                                                                              \
  do {                                                                                     \
    cudaError_t e_ = (x);                                                                  \
    if (e_ != cudaSuccess) {                                                               \
      fc3dgpu_set_error("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
      return NUMERICS_ERR_UNKNOWN;                                                         \
    }                                                                                      \
  } while (0)

template <typename T>
static cudaError_t ensure(T** p, size_t* cap, size_t n) {
  if (*p && *cap >= n) return cudaSuccess;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc((void**)p, (n ? n : 1) * sizeof(T));
  if (e == cudaSuccess) *cap = n;
  return e;
}

#define BUF(T, name) \
  T* name = nullptr; \
  size_t name##_cap = 0

struct fc3dgpu_ctx {
  int device = 0;
  int nsm = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  int nc = 0;
  long long nnzb = 0;
  int ncol = 0, nslab = 0, npad = 0;
  long long nslots = 0;
  int sptr[FC3D_MAX_COLOURS + 1];
  double norm_q = 0.0;
  bool have_W = false, have_q = false, have_r = false;
  int trace_len = 0;
  // inputs (original order)
  BUF(long long, rowptr);
  BUF(long long, colidx);
  BUF(double, blocks);
  BUF(double, qo);
  BUF(double, muo);
  BUF(double, ro);
  BUF(double, uo);
  // colouring
  BUF(int, deg);
  BUF(long long, gptr64);
  BUF(int, gptr);
  BUF(int, cursor);
  BUF(int, adj);
  BUF(uint32_t, key);
  BUF(int, colour);
  BUF(int, blockhist);
  BUF(int, counts);
  BUF(int, sptr_d);
  // layout
  BUF(int, perm);
  BUF(int, iperm);
  BUF(int, rowlen);
  BUF(int, dpos);
  BUF(int, slab_nslot);
  BUF(long long, slab_off);
  BUF(double, W64);
  BUF(float, W32);
  BUF(int, col);
  BUF(double, D64);
  BUF(float, D32);
  BUF(double, rho64);
  BUF(float, rho32);
  BUF(double, q64);
  BUF(float, q32);
  BUF(double, mu64);
  BUF(float, mu32);
  BUF(double, r64);
  BUF(float, r32);
  BUF(double, rpli64);
  BUF(float, rpli32);
  BUF(double, u64);
  // control
  BUF(double, partials);
  BUF(unsigned, barrier);
  BUF(int, status);
  BUF(int, scratch);
  BUF(long long, scratch64);
  BUF(double, out);
  BUF(double, trace);
  BUF(unsigned long long, counters);
  int counters_on = 0;
  unsigned long long launches = 0;  // kernels this library launched
  BUF(unsigned long long, timeline);
  int timeline_sweep = 0;
  std::vector<long long> slab_off_h;
  int ccount[FC3D_MAX_COLOURS];
  std::vector<int> slab_nslot_h;
  int staging = 1;  // bulk-copy staging of slab ranges for the FP32 sweeps
  unsigned long long spin_limit = 0;  // polls before a device wait gives up (0: 2^22)
  // slab-dataflow FP32 sweep: on/off, and its per-layout column lists
  // (state 0: not built for this layout, 1: built, -1: does not apply)
  int flow_on = 1;
  int flow_state = 0;
  int flow_nw = 0, flow_maxslot = 0;
  int flow_want = 0;  // warps per block of the dataflow sweep asked for (0: default)
  // measuring autotuner (per layout): chosen FP32 variant and FP64 lanes,
  // and the measured device time of one sweep of every candidate
  int tuned = 0;          // 0: not yet for this layout
  int tune_mode = 1;      // 0 off, 1 result-preserving variants only, 2 every variant
  int tune_flow = 0, tune_nw = 0, tune_lanes32 = 1, tune_lanes64 = 1;
  float tune_ms32[7] = {0}, tune_ms64[4] = {0};
  BUF(double, tune_r64);
  BUF(double, tune_rpli64);
  BUF(float, tune_rpli32);
  BUF(int, flow_dptr);
  BUF(int, flow_dep);
  BUF(unsigned, flow_done);
  BUF(int2, flow_need);
  BUF(int, flow_sptr);
  BUF(double, flow_part);
  BUF(long long, flow_rec_off);
  BUF(float, flow_rec);
  // batched problems (0 = a single problem)
  int nscenes = 0;
  std::vector<int> scene_off_h;  // nscenes + 1 contact offsets
  std::vector<double> scene_normq_h;
  BUF(int, scene_off);
  BUF(int, grp);
  BUF(int, scounts);
  BUF(int, snslab);
  BUF(int, sncol);
  BUF(long long, sbase);
  BUF(int, ssptr);
  BUF(int, sorder);
  BUF(double, snormq);
  BUF(int, sbudget);
  BUF(int, squeue);
  BUF(double, sout32);
  BUF(double, sout64);
  cudaGraphExec_t batch_graph = nullptr;
  fc3dgpu_params batch_graph_params;
  // resident blocks of the batched kernels (FP32, FP64, fast FP64), set before capture
  int batch_grid32 = 0, batch_grid64 = 0, batch_grid64f = 0;
  // neighbourhood synchronisation: block neighbour lists per grid size
  struct Nbr {
    int grid = 0;
    int* ptr = nullptr;
    int* list = nullptr;
  } nbrc[2];
  int nbr_next = 0;
  BUF(unsigned, nbrmask);
  int nbr_sync = 1;  // neighbourhood synchronisation on (1, default) or grid barriers (0)
  int colour_kind = -1;  // colouring of the current layout
  BUF(long long, wtmp);  // new structure for a comparison with the current one
  BUF(int, wdiff);
  // upload of W's values through block pointers: per host thread a stream,
  // two pinned staging buffers for scattered blocks with their copy events,
  // and an event closing the thread's copies
  cudaStream_t up_stream[4] = {nullptr, nullptr, nullptr, nullptr};
  double* up_stage[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t up_ev[4][2] = {};
  cudaEvent_t up_done[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t up_start = nullptr;
  int* diff_h = nullptr;  // pinned: the structure comparison's result
  // device assembly of W and q from rigid-body contacts
  int nb = 0;
  double step_h = 0.0;
  bool have_contacts = false, have_mu = false, have_vel = false;
  BUF(int, cbA);
  BUF(int, cbB);
  BUF(double, cframe);
  BUF(double, cpoint);
  BUF(double, bpos);
  BUF(double, bmass);
  BUF(double, binert);
  BUF(double, bvel);
  BUF(int, bdeg);
  BUF(long long, bptr);
  BUF(int, blist);
  BUF(int, crowlen);
  BUF(double, qsum);
  // learned warm start
  BUF(float, feat);
  BUF(float, prop);
  BUF(double, rbak);
  BUF(double, gapo);
};

static int grid1d(long long n, int block = 256) {
  long long g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > 65535LL * 8) g = 65535LL * 8;
  return (int)g;
}

extern "C" void fc3dgpu_params_default(fc3dgpu_params* p) {
  p->tol = 1e-4;
  p->max_iter = 1000;
  p->precision = 0;
  p->lanes = 0;
  p->switch_tol = 1e-6;
  p->stall_window = 64;
  p->local_tol = 1e-14;
  // FP32 local tolerance: 1e-6 sits a few FP32 ulps above the resolution of
  // the relative local error, so Newton often cannot certify it and falls to
  // PLI; 1e-5 gives the same progress per sweep (60x60x30 lattice: the same
  // light error after 100 sweeps to 4 digits, the same 550 sweeps to 1e-3)
  // for 3 % less time per sweep
  p->local_tol32 = 1e-5;
  p->newton_max = 100;
  p->pli_max = 100;
  p->ls_max = 10;
  p->local_mode32 = 0;
  p->fp32_only = 0;
  p->relax = 0;
  p->omega = 1.0;
  p->filter = 0;
}

extern "C" fc3dgpu_ctx* fc3dgpu_ctx_create(int device) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n <= device || device < 0) {
    fc3dgpu_set_error("no CUDA device %d (%s)", device, e != cudaSuccess ? cudaGetErrorString(e) : "count");
    return nullptr;
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    fc3dgpu_set_error("cudaSetDevice(%d) failed", device);
    return nullptr;
  }
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  if (!coop) {
    fc3dgpu_set_error("device %d does not support cooperative launches", device);
    return nullptr;
  }
  fc3dgpu_ctx* c = new fc3dgpu_ctx();
  c->device = device;
  cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    fc3dgpu_set_error("cudaStreamCreate failed");
    return nullptr;
  }
  for (int i = 0; i < 4; i++) cudaEventCreate(&c->ev[i]);
  // load every sweep kernel now: with lazy module loading the first launch
  // of each instance would otherwise pay the load inside a timed solve
  fc3dgpu::warm_sweep_kernels();
  fc3dgpu::warm_batch_kernel_f32();
  fc3dgpu::warm_batch_kernel_f64();
  bool ok = ensure(&c->partials, &c->partials_cap, 1024 * 8) == cudaSuccess &&
            ensure(&c->barrier, &c->barrier_cap, FC3D_BARRIER_WORDS) == cudaSuccess &&
            ensure(&c->status, &c->status_cap, 4) == cudaSuccess &&
            ensure(&c->scratch, &c->scratch_cap, 16) == cudaSuccess &&
            ensure(&c->scratch64, &c->scratch64_cap, 16) == cudaSuccess &&
            ensure(&c->out, &c->out_cap, 16) == cudaSuccess &&
            ensure(&c->trace, &c->trace_cap, 1 << 17) == cudaSuccess &&
            ensure(&c->counters, &c->counters_cap, 8) == cudaSuccess;
  if (!ok) {
    fc3dgpu_set_error("device allocation failed");
    fc3dgpu_ctx_destroy(c);
    return nullptr;
  }
  return c;
}

extern "C" void fc3dgpu_ctx_destroy(fc3dgpu_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  void* ptrs[] = {c->rowptr, c->colidx, c->blocks, c->qo, c->muo, c->ro, c->uo, c->deg, c->gptr64, c->gptr,
                  c->cursor, c->adj, c->key, c->colour, c->blockhist, c->counts, c->sptr_d, c->perm, c->iperm,
                  c->rowlen, c->dpos, c->slab_nslot, c->slab_off, c->W64, c->W32, c->col, c->D64, c->D32,
                  c->rho64, c->rho32, c->q64, c->q32, c->mu64, c->mu32, c->r64, c->r32, c->rpli64, c->rpli32,
                  c->u64, c->partials, c->barrier, c->status, c->scratch, c->scratch64, c->out, c->trace,
                  c->counters, c->timeline, c->scene_off, c->grp, c->scounts, c->snslab, c->sncol, c->sbase,
                  c->ssptr, c->sorder, c->snormq, c->sbudget, c->squeue, c->sout32, c->sout64, c->feat,
                  c->prop, c->rbak, c->gapo, c->cbA, c->cbB, c->cframe, c->cpoint, c->bpos, c->bmass,
                  c->binert, c->bvel, c->bdeg, c->bptr, c->blist, c->crowlen, c->qsum, c->wtmp, c->wdiff,
                  c->flow_dptr, c->flow_dep, c->flow_done, c->flow_need, c->flow_sptr, c->flow_part,
                  c->flow_rec_off, c->flow_rec};
  if (c->batch_graph) cudaGraphExecDestroy(c->batch_graph);
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (auto& n : c->nbrc) {
    if (n.ptr) cudaFree(n.ptr);
    if (n.list) cudaFree(n.list);
  }
  if (c->nbrmask) cudaFree(c->nbrmask);
  for (int i = 0; i < 4; i++)
    if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  for (int t = 0; t < 4; t++) {
    for (int i = 0; i < 2; i++)
      if (c->up_ev[t][i]) cudaEventDestroy(c->up_ev[t][i]);
    if (c->up_done[t]) cudaEventDestroy(c->up_done[t]);
    if (c->up_stage[t]) cudaFreeHost(c->up_stage[t]);
    if (c->up_stream[t]) cudaStreamDestroy(c->up_stream[t]);
  }
  if (c->up_start) cudaEventDestroy(c->up_start);
  if (c->diff_h) cudaFreeHost(c->diff_h);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

// Host check of a block-CSR structure before any device kernel indexes with
// it: monotone row pointer, column indices inside [0, nc).
static int validate_bcsr(int nc, const int64_t* rowptr, const int64_t* colidx) {
  if (rowptr[0] != 0) {
    fc3dgpu_set_error("row pointer must start at 0");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  for (int i = 0; i < nc; i++) {
    if (rowptr[i + 1] < rowptr[i]) {
      fc3dgpu_set_error("row pointer decreases at row %d", i);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++)
      if (colidx[k] < 0 || colidx[k] >= nc) {
        fc3dgpu_set_error("block column %lld out of range in row %d", (long long)colidx[k], i);
        return NUMERICS_ERR_INVALID_ARGUMENT;
      }
  }
  return 0;
}

// Colour the conflict graph of the uploaded structure (rowptr/colidx on the
// device); result in c->colour, number of colours returned.
static int colour_device(fc3dgpu_ctx* c, int nc, long long nnzb, int kind, const int* grp = nullptr,
                         const int* group_off = nullptr) {
  using namespace fc3dgpu;
  cudaStream_t s = c->stream;
  CK(ensure(&c->deg, &c->deg_cap, (size_t)nc));
  CK(ensure(&c->gptr64, &c->gptr64_cap, (size_t)nc + 1));
  CK(ensure(&c->gptr, &c->gptr_cap, (size_t)nc + 1));
  CK(ensure(&c->cursor, &c->cursor_cap, (size_t)nc));
  CK(ensure(&c->key, &c->key_cap, (size_t)nc));
  CK(ensure(&c->colour, &c->colour_cap, (size_t)nc));
  CK(cudaMemsetAsync(c->deg, 0, sizeof(int) * nc, s));
  k_degree<<<grid1d(nc), 256, 0, s>>>(nc, c->rowptr, c->colidx, c->deg);
  k_scan_excl<int><<<1, 1024, 0, s>>>(nc, c->deg, c->gptr64, c->scratch64);
  long long nadj = 0;
  CK(cudaMemcpyAsync(&nadj, c->scratch64, sizeof(long long), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (nadj > 0x7fffffffLL) {
    fc3dgpu_set_error("conflict graph too large (%lld entries)", nadj);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  CK(cudaMemcpyAsync(c->gptr64 + nc, c->scratch64, sizeof(long long), cudaMemcpyDeviceToDevice, s));
  k_ll_to_int<<<grid1d(nc + 1), 256, 0, s>>>(nc + 1, c->gptr64, c->gptr);
  CK(ensure(&c->adj, &c->adj_cap, (size_t)(nadj ? nadj : 1)));
  CK(cudaMemcpyAsync(c->cursor, c->gptr, sizeof(int) * nc, cudaMemcpyDeviceToDevice, s));
  k_adjacency<<<grid1d(nc), 256, 0, s>>>(nc, c->rowptr, c->colidx, c->cursor, c->adj);
  const int passes = (kind >> 8) & 0xff;
  const bool kempe = (kind & FC3DGPU_COLOUR_KEMPE) != 0;
  kind &= 0xff;
  k_priority<<<grid1d(nc), 256, 0, s>>>(nc, c->gptr, c->adj, kind, c->key, c->colour, grp, group_off);
  int ncol = 0;
  for (int pass = 0; pass <= passes; pass++) {
    if (pass > 0)
      k_recolour_key<<<grid1d(nc), 256, 0, s>>>(nc, grp, group_off, c->key, c->colour);
    int rounds = 0;
    for (;;) {
      CK(cudaMemsetAsync(c->scratch, 0, 2 * sizeof(int), s));
      k_jp_round<<<grid1d(nc), 256, 0, s>>>(nc, c->gptr, c->adj, c->key, c->colour, c->scratch, c->scratch + 1);
      int h[2];
      CK(cudaMemcpyAsync(h, c->scratch, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      if (h[1]) {
        fc3dgpu_set_error("colouring needs more than %d colours", FC3D_MAX_COLOURS);
        return NUMERICS_ERR_INVALID_ARGUMENT;
      }
      if (h[0] == 0) break;
      if (++rounds > nc + 1) {
        fc3dgpu_set_error("colouring did not finish");
        return NUMERICS_ERR_UNKNOWN;
      }
    }
    CK(cudaMemsetAsync(c->scratch + 2, 0xff, sizeof(int), s));
    k_max_colour<<<grid1d(nc), 256, 0, s>>>(nc, c->colour, c->scratch + 2);
    int mx = -1;
    CK(cudaMemcpyAsync(&mx, c->scratch + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    ncol = mx + 1;
  }
  if (kempe && ncol > 1) {
    // Kempe-chain reduction on the host (deterministic: it does not depend
    // on the order of the adjacency lists the device wrote)
    std::vector<int> gptr((size_t)nc + 1), adj((size_t)(nadj ? nadj : 1)), col((size_t)nc);
    CK(cudaMemcpyAsync(gptr.data(), c->gptr, sizeof(int) * (nc + 1), cudaMemcpyDeviceToHost, s));
    if (nadj) CK(cudaMemcpyAsync(adj.data(), c->adj, sizeof(int) * nadj, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(col.data(), c->colour, sizeof(int) * nc, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (!grp) {
      const int n = fc3dgpu_colour_reduce(nc, gptr.data(), adj.data(), col.data(), ncol, 0);
      if (n > 0) ncol = n;
    } else {
      // each problem on its own (its rows only meet its own rows), so it
      // gets the colouring it would get alone; the problems on the host's
      // threads
      const int ng = (int)c->scene_off_h.size() - 1;
      const int nth = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), 16u);
      const int r = fc3dgpu_colour_reduce_groups(ng, c->scene_off_h.data(), gptr.data(), adj.data(), col.data(), nth);
      if (r > 0) ncol = r;
    }
    CK(cudaMemcpyAsync(c->colour, col.data(), sizeof(int) * nc, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
  }
  return ncol;
}

static int build_layout(fc3dgpu_ctx* c, int nc, long long nnzb, int kind, int nscenes, const int* scene_nc);

// The values of W: one array of nnzb column-major 3x3 blocks (flat), or one
// pointer per block (ptrs[k] -> 9 doubles), the layout of the block array of
// a SparseBlockStructuredMatrix (SparseBlockMatrix.h, block[k]).
struct BlockSource {
  const double* flat;
  const double* const* ptrs;
};

// Blocks per step of upload_blocks (one copy each), and the host threads
// that take the steps in turn.
static const long long STAGE_BLOCKS = 1 << 16;
static const int UPLOAD_THREADS = 4;

// Copy nnzb blocks from src into c->blocks (stream-ordered on c->stream).
// From a block pointer array, up to four host threads take the steps of
// STAGE_BLOCKS blocks in turn, each on its own stream: a step whose blocks
// lie back to back in memory is copied straight from there, another one is
// gathered into one of the thread's two pinned staging buffers first.
static int upload_blocks(fc3dgpu_ctx* c, long long nnzb, BlockSource src) {
  cudaStream_t s = c->stream;
  if (src.flat) {
    CK(cudaMemcpyAsync(c->blocks, src.flat, sizeof(double) * 9 * nnzb, cudaMemcpyHostToDevice, s));
    return 0;
  }
  const double* const* p = src.ptrs;
  const long long nstep = (nnzb + STAGE_BLOCKS - 1) / STAGE_BLOCKS;
  const int nth = nstep >= 8 ? UPLOAD_THREADS : 1;
  if (!c->up_start) CK(cudaEventCreateWithFlags(&c->up_start, cudaEventDisableTiming));
  for (int t = 0; t < nth; t++) {
    if (!c->up_stream[t]) CK(cudaStreamCreateWithFlags(&c->up_stream[t], cudaStreamNonBlocking));
    if (!c->up_done[t]) CK(cudaEventCreateWithFlags(&c->up_done[t], cudaEventDisableTiming));
    for (int i = 0; i < 2; i++)
      if (!c->up_ev[t][i]) CK(cudaEventCreateWithFlags(&c->up_ev[t][i], cudaEventDisableTiming));
  }
  // the copies follow whatever the context's stream already holds
  CK(cudaEventRecord(c->up_start, s));
  std::atomic<int> failed{0};           // 1: a null block pointer, 2: a CUDA call failed
  std::atomic<long long> null_at{-1};
  std::atomic<int> cuda_err{0};
  auto worker = [&](int t) {
    auto ok = [&](cudaError_t e) {
      if (e == cudaSuccess) return true;
      cuda_err.store((int)e);
      failed.store(2);
      return false;
    };
    if (!ok(cudaSetDevice(c->device)) || !ok(cudaStreamWaitEvent(c->up_stream[t], c->up_start, 0))) return;
    const uintptr_t bsz = sizeof(double) * 9;
    int slot = 0;
    for (long long st = t; st < nstep && !failed.load(std::memory_order_relaxed); st += nth) {
      const long long k0 = st * STAGE_BLOCKS, k1 = k0 + STAGE_BLOCKS < nnzb ? k0 + STAGE_BLOCKS : nnzb;
      const uintptr_t b0 = (uintptr_t)p[k0];
      uintptr_t off = 0;
      for (long long k = k0; k < k1; k++) off |= (uintptr_t)p[k] ^ (b0 + bsz * (uintptr_t)(k - k0));
      if (b0 != 0 && off == 0) {
        if (!ok(cudaMemcpyAsync(c->blocks + 9 * k0, p[k0], sizeof(double) * 9 * (k1 - k0), cudaMemcpyHostToDevice,
                                c->up_stream[t])))
          return;
        continue;
      }
      // scattered blocks: into a staging buffer once its last copy is done
      if (!c->up_stage[t] &&
          !ok(cudaHostAlloc((void**)&c->up_stage[t], sizeof(double) * 9 * 2 * STAGE_BLOCKS, cudaHostAllocDefault)))
        return;
      if (!ok(cudaEventSynchronize(c->up_ev[t][slot]))) return;
      double* buf = c->up_stage[t] + 9 * STAGE_BLOCKS * slot;
      for (long long k = k0; k < k1; k++) {
        if (!p[k]) {
          null_at.store(k);
          failed.store(1);
          return;
        }
        memcpy(buf + 9 * (k - k0), p[k], sizeof(double) * 9);
      }
      if (!ok(cudaMemcpyAsync(c->blocks + 9 * k0, buf, sizeof(double) * 9 * (k1 - k0), cudaMemcpyHostToDevice,
                              c->up_stream[t])) ||
          !ok(cudaEventRecord(c->up_ev[t][slot], c->up_stream[t])))
        return;
      slot ^= 1;
    }
  };
  {
    std::vector<std::thread> th;
    int started = 1;
    try {
      for (int t = 1; t < nth; t++) {
        th.emplace_back(worker, t);
        started++;
      }
    } catch (...) {
      // fewer threads to be had: the rest run here
    }
    worker(0);
    for (int t = started; t < nth; t++) worker(t);
    for (auto& x : th) x.join();
  }
  // the context's stream waits for every thread's copies
  for (int t = 0; t < nth; t++) {
    CK(cudaEventRecord(c->up_done[t], c->up_stream[t]));
    CK(cudaStreamWaitEvent(s, c->up_done[t], 0));
  }
  if (failed.load()) {
    CK(cudaStreamSynchronize(s));
    if (failed.load() == 2) {
      fc3dgpu_set_error("CUDA error %d (%s) in the upload of W", cuda_err.load(),
                        cudaGetErrorString((cudaError_t)cuda_err.load()));
      return NUMERICS_ERR_UNKNOWN;
    }
    fc3dgpu_set_error("block %lld of W is a null pointer", null_at.load());
    return NUMERICS_ERR_NULL_POINTER;
  }
  return 0;
}

static int set_W_impl(fc3dgpu_ctx* c, int nc, const int64_t* rowptr, const int64_t* colidx, BlockSource blocks,
                      int kind, int nscenes, const int* scene_nc) {
  using namespace fc3dgpu;
  if (!c || nc <= 0 || !rowptr || !colidx || (!blocks.flat && !blocks.ptrs)) {
    fc3dgpu_set_error("fc3dgpu_ctx_set_W: invalid argument");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  CK(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  const long long nnzb = rowptr[nc];
  if (nnzb < nc) {
    fc3dgpu_set_error("fc3dgpu_ctx_set_W: fewer blocks than block rows");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  {
    int v = validate_bcsr(nc, rowptr, colidx);
    if (v) return v;
  }
  c->have_W = c->have_q = c->have_r = false;
  c->have_contacts = c->have_vel = c->have_mu = false;  // W no longer comes from contact geometry
  CK(ensure(&c->rowptr, &c->rowptr_cap, (size_t)nc + 1));
  CK(ensure(&c->colidx, &c->colidx_cap, (size_t)nnzb));
  CK(ensure(&c->blocks, &c->blocks_cap, (size_t)nnzb * 9));
  CK(cudaMemcpyAsync(c->rowptr, rowptr, sizeof(long long) * (nc + 1), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->colidx, colidx, sizeof(long long) * nnzb, cudaMemcpyHostToDevice, s));
  {
    int rc = upload_blocks(c, nnzb, blocks);
    if (rc) return rc;
  }
  return build_layout(c, nc, nnzb, kind, nscenes, scene_nc);
}

// Colouring, permutation and slab layout of the block-CSR W already in
// c->rowptr, c->colidx, c->blocks (original contact order).
static int build_layout(fc3dgpu_ctx* c, int nc, long long nnzb, int kind, int nscenes, const int* scene_nc) {
  using namespace fc3dgpu;
  cudaStream_t s = c->stream;
  c->have_W = c->have_q = c->have_r = false;
  c->nscenes = nscenes;
  const int* d_grp = nullptr;
  if (nscenes > 0) {
    c->scene_off_h.assign(nscenes + 1, 0);
    for (int g = 0; g < nscenes; g++) c->scene_off_h[g + 1] = c->scene_off_h[g] + scene_nc[g];
    if (c->scene_off_h[nscenes] != nc) {
      fc3dgpu_set_error("problem sizes add up to %d contacts, W has %d", c->scene_off_h[nscenes], nc);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
    CK(ensure(&c->scene_off, &c->scene_off_cap, (size_t)nscenes + 1));
    CK(ensure(&c->grp, &c->grp_cap, (size_t)nc));
    CK(cudaMemcpyAsync(c->scene_off, c->scene_off_h.data(), sizeof(int) * (nscenes + 1), cudaMemcpyHostToDevice, s));
    k_group_ids<<<nscenes, 256, 0, s>>>(nscenes, c->scene_off, c->grp);
    d_grp = c->grp;
  }
  int ncol = colour_device(c, nc, nnzb, kind, d_grp, nscenes > 0 ? c->scene_off : nullptr);
  if (ncol < 0) return ncol;
  const int nblk = (nc + 1023) / 1024;
  CK(ensure(&c->counts, &c->counts_cap, FC3D_MAX_COLOURS));
  CK(ensure(&c->sptr_d, &c->sptr_d_cap, FC3D_MAX_COLOURS + 1));
  if (nscenes == 0) {
    // stable permutation by colour
    CK(ensure(&c->blockhist, &c->blockhist_cap, (size_t)nblk * FC3D_MAX_COLOURS));
    k_colour_hist<<<nblk, 1024, 0, s>>>(nc, c->colour, c->blockhist);
    k_colour_offsets<<<1, FC3D_MAX_COLOURS, 0, s>>>(nblk, c->blockhist, c->counts, c->sptr_d);
    CK(cudaMemcpyAsync(c->sptr, c->sptr_d, sizeof(int) * (FC3D_MAX_COLOURS + 1), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(c->ccount, c->counts, sizeof(int) * FC3D_MAX_COLOURS, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    c->ncol = ncol;
    c->nslab = c->sptr[ncol];
  } else {
    // per problem, stable permutation by colour; problems one after the other
    CK(ensure(&c->scounts, &c->scounts_cap, (size_t)nscenes * FC3D_MAX_COLOURS));
    CK(ensure(&c->snslab, &c->snslab_cap, (size_t)nscenes));
    CK(ensure(&c->sncol, &c->sncol_cap, (size_t)nscenes));
    CK(ensure(&c->sbase, &c->sbase_cap, (size_t)nscenes));
    CK(ensure(&c->ssptr, &c->ssptr_cap, (size_t)nscenes * (FC3D_MAX_COLOURS + 1)));
    k_scene_counts<<<nscenes, 256, 0, s>>>(c->scene_off, c->colour, c->scounts, c->snslab, c->sncol);
    k_scan_excl<int><<<1, 1024, 0, s>>>(nscenes, c->snslab, c->sbase, c->scratch64);
    long long tot = 0;
    CK(cudaMemcpyAsync(&tot, c->scratch64, sizeof(long long), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    c->ncol = ncol;
    c->nslab = (int)tot;
    for (int k = 0; k <= FC3D_MAX_COLOURS; k++) c->sptr[k] = k ? c->nslab : 0;
    for (int k = 0; k < FC3D_MAX_COLOURS; k++) c->ccount[k] = 0;
  }
  c->npad = c->nslab * FC3D_SLAB;
  const int npad = c->npad, nslab = c->nslab;
  CK(ensure(&c->perm, &c->perm_cap, (size_t)npad));
  CK(ensure(&c->iperm, &c->iperm_cap, (size_t)nc));
  CK(cudaMemsetAsync(c->perm, 0xff, sizeof(int) * npad, s));
  if (nscenes == 0) {
    k_colour_scatter<<<nblk, 1024, 0, s>>>(nc, c->colour, c->blockhist, c->sptr_d, c->perm, c->iperm);
  } else {
    k_scene_scatter<<<nscenes, 1024, 0, s>>>(c->scene_off, c->colour, c->scounts, c->sbase, c->ssptr, c->perm,
                                             c->iperm);
    // problems by decreasing size for the work queue
    std::vector<int> order(nscenes);
    for (int g = 0; g < nscenes; g++) order[g] = g;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return scene_nc[x] > scene_nc[y]; });
    CK(ensure(&c->sorder, &c->sorder_cap, (size_t)nscenes));
    CK(cudaMemcpyAsync(c->sorder, order.data(), sizeof(int) * nscenes, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
  }
  // rows, slabs, slots
  CK(ensure(&c->rowlen, &c->rowlen_cap, (size_t)npad));
  CK(ensure(&c->dpos, &c->dpos_cap, (size_t)npad));
  CK(ensure(&c->slab_nslot, &c->slab_nslot_cap, (size_t)nslab));
  CK(ensure(&c->slab_off, &c->slab_off_cap, (size_t)nslab));
  CK(cudaMemsetAsync(c->scratch + 3, 0, sizeof(int), s));
  k_rowinfo<<<grid1d(npad), 256, 0, s>>>(npad, c->perm, c->rowptr, c->colidx, c->rowlen, c->dpos, c->scratch + 3);
  k_slab_nslot<<<grid1d((long long)nslab * 32), 256, 0, s>>>(nslab, c->rowlen, c->slab_nslot);
  k_scan_excl<int><<<1, 1024, 0, s>>>(nslab, c->slab_nslot, c->slab_off, c->scratch64);
  long long nslots = 0;
  int nodiag = 0;
  CK(cudaMemcpyAsync(&nslots, c->scratch64, sizeof(long long), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&nodiag, c->scratch + 3, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (nodiag) {
    fc3dgpu_set_error("W has a block row without its diagonal block");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  c->nslots = nslots;
  c->slab_off_h.resize(nslab);
  c->slab_nslot_h.resize(nslab);
  CK(cudaMemcpyAsync(c->slab_off_h.data(), c->slab_off, sizeof(long long) * nslab, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(c->slab_nslot_h.data(), c->slab_nslot, sizeof(int) * nslab, cudaMemcpyDeviceToHost, s));
  const size_t nw = (size_t)(nslots ? nslots : 1) * 9 * FC3D_SLAB;
  CK(ensure(&c->W64, &c->W64_cap, nw));
  CK(ensure(&c->W32, &c->W32_cap, nw));
  CK(ensure(&c->col, &c->col_cap, (size_t)(nslots ? nslots : 1) * FC3D_SLAB));
  CK(ensure(&c->D64, &c->D64_cap, (size_t)nslab * 9 * FC3D_SLAB));
  CK(ensure(&c->D32, &c->D32_cap, (size_t)nslab * 9 * FC3D_SLAB));
  CK(ensure(&c->rho64, &c->rho64_cap, (size_t)nslab * 2 * FC3D_SLAB));
  CK(ensure(&c->rho32, &c->rho32_cap, (size_t)nslab * 2 * FC3D_SLAB));
  CK(ensure(&c->q64, &c->q64_cap, (size_t)nslab * 3 * FC3D_SLAB));
  CK(ensure(&c->q32, &c->q32_cap, (size_t)nslab * 3 * FC3D_SLAB));
  CK(ensure(&c->mu64, &c->mu64_cap, (size_t)npad));
  CK(ensure(&c->mu32, &c->mu32_cap, (size_t)npad));
  CK(ensure(&c->r64, &c->r64_cap, ((size_t)npad + 1) * 4));
  CK(ensure(&c->r32, &c->r32_cap, ((size_t)npad + 1) * 4));
  CK(ensure(&c->rpli64, &c->rpli64_cap, (size_t)npad));
  CK(ensure(&c->rpli32, &c->rpli32_cap, (size_t)npad));
  CK(ensure(&c->u64, &c->u64_cap, (size_t)npad * 3));
  CK(cudaMemsetAsync(c->W64, 0, sizeof(double) * nw, s));
  CK(cudaMemsetAsync(c->D64, 0, sizeof(double) * nslab * 9 * FC3D_SLAB, s));
  CK(cudaMemsetAsync(c->rho64, 0, sizeof(double) * nslab * 2 * FC3D_SLAB, s));
  CK(cudaMemsetAsync(c->q64, 0, sizeof(double) * nslab * 3 * FC3D_SLAB, s));
  CK(cudaMemsetAsync(c->q32, 0, sizeof(float) * nslab * 3 * FC3D_SLAB, s));
  CK(cudaMemsetAsync(c->mu64, 0, sizeof(double) * npad, s));
  CK(cudaMemsetAsync(c->mu32, 0, sizeof(float) * npad, s));
  CK(cudaMemsetAsync(c->r64, 0, sizeof(double) * (npad + 1) * 4, s));
  CK(cudaMemsetAsync(c->r32, 0, sizeof(float) * (npad + 1) * 4, s));
  CK(cudaMemsetAsync(c->u64, 0, sizeof(double) * npad * 3, s));
  k_fill_col_pad<<<grid1d((long long)nslots * FC3D_SLAB), 256, 0, s>>>(nslots, npad, c->col);
  k_fill_blocks<<<grid1d(npad, 128), 128, 0, s>>>(npad, c->perm, c->rowptr, c->colidx, c->blocks, c->iperm,
                                                  c->slab_off, c->W64, c->col, c->D64, c->rho64);
  k_to_f32<<<grid1d((long long)nw), 256, 0, s>>>((long long)nw, c->W64, c->W32);
  k_to_f32<<<grid1d((long long)nslab * 9 * 32), 256, 0, s>>>((long long)nslab * 9 * 32, c->D64, c->D32);
  k_to_f32<<<grid1d((long long)nslab * 2 * 32), 256, 0, s>>>((long long)nslab * 2 * 32, c->rho64, c->rho32);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  c->nc = nc;
  c->nnzb = nnzb;
  c->have_W = true;
  c->colour_kind = kind;
  for (auto& n : c->nbrc) n.grid = 0;  // the rows' owners changed
  c->flow_state = 0;
  c->tuned = 0;
  return 0;
}

extern "C" int fc3dgpu_ctx_set_W(fc3dgpu_ctx* c, int nc, const int64_t* rowptr, const int64_t* colidx,
                                 const double* blocks, int kind) {
  if (c && c->batch_graph) {
    cudaGraphExecDestroy(c->batch_graph);
    c->batch_graph = nullptr;
  }
  return set_W_impl(c, nc, rowptr, colidx, BlockSource{blocks, nullptr}, kind, 0, nullptr);
}

// Many independent problems as one block-diagonal W: the union block-CSR
// (problem k's rows and columns are contacts scene_off[k] ..), nscenes and
// each problem's contact count.
extern "C" int fc3dgpu_ctx_set_W_batch(fc3dgpu_ctx* c, int nscenes, const int* scene_nc, const int64_t* rowptr,
                                       const int64_t* colidx, const double* blocks, int kind) {
  if (!c || nscenes <= 0 || !scene_nc) {
    fc3dgpu_set_error("fc3dgpu_ctx_set_W_batch: invalid argument");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  long long nc = 0;
  for (int k = 0; k < nscenes; k++) {
    if (scene_nc[k] <= 0) {
      fc3dgpu_set_error("problem %d has no contact", k);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
    nc += scene_nc[k];
  }
  if (nc > 0x7fffffffLL) {
    fc3dgpu_set_error("too many contacts in the batch");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  // a block of W must not join two problems
  long long off = 0;
  for (int k = 0; k < nscenes; k++) {
    for (long long i = off; i < off + scene_nc[k]; i++)
      for (int64_t kk = rowptr[i]; kk < rowptr[i + 1]; kk++)
        if (colidx[kk] < off || colidx[kk] >= off + scene_nc[k]) {
          fc3dgpu_set_error("W couples problem %d to another problem (row %lld)", k, i);
          return NUMERICS_ERR_INVALID_ARGUMENT;
        }
    off += scene_nc[k];
  }
  if (c->batch_graph) {
    cudaGraphExecDestroy(c->batch_graph);
    c->batch_graph = nullptr;
  }
  if (!blocks) {
    fc3dgpu_set_error("fc3dgpu_ctx_set_W_batch: invalid argument");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  return set_W_impl(c, (int)nc, rowptr, colidx, BlockSource{blocks, nullptr}, kind, nscenes, scene_nc);
}

// |q| of 3nc doubles: four interleaved partial sums of squares combined in a
// fixed order (deterministic; a plain index-order sum would be a 3nc-long
// dependent chain).
extern "C" double fc3dgpu_norm_q_host(const double* q, long long n) {
  double s4[4] = {0.0, 0.0, 0.0, 0.0};
  long long i = 0;
  for (; i + 4 <= n; i += 4)
    for (int k = 0; k < 4; k++) s4[k] += q[i + k] * q[i + k];
  for (; i < n; i++) s4[0] += q[i] * q[i];
  return sqrt((s4[0] + s4[1]) + (s4[2] + s4[3]));
}

static int set_q_mu_impl(fc3dgpu_ctx* c, const double* q, const double* mu, double norm_q);

extern "C" int fc3dgpu_ctx_set_q_mu(fc3dgpu_ctx* c, const double* q, const double* mu) {
  return set_q_mu_impl(c, q, mu, -1.0);
}

// fc3dgpu_ctx_set_q_mu with |q| computed by the caller (fc3dgpu_norm_q_host)
extern "C" int fc3dgpu_ctx_set_q_mu_norm(fc3dgpu_ctx* c, const double* q, const double* mu, double norm_q) {
  return set_q_mu_impl(c, q, mu, norm_q);
}

static int set_q_mu_impl(fc3dgpu_ctx* c, const double* q, const double* mu, double norm_q) {
  using namespace fc3dgpu;
  if (!c || !c->have_W || !q || !mu) {
    fc3dgpu_set_error("fc3dgpu_ctx_set_q_mu: W not set or null input");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  CK(cudaSetDevice(c->device));
  const int nc = c->nc;
  CK(ensure(&c->qo, &c->qo_cap, (size_t)nc * 3));
  CK(ensure(&c->muo, &c->muo_cap, (size_t)nc));
  CK(cudaMemcpyAsync(c->qo, q, sizeof(double) * 3 * nc, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->muo, mu, sizeof(double) * nc, cudaMemcpyHostToDevice, c->stream));
  k_set_q_mu<<<grid1d(nc), 256, 0, c->stream>>>(nc, c->iperm, c->qo, c->muo, c->q64, c->mu64, c->q32, c->mu32);
  CK(cudaGetLastError());
  c->launches++;
  // |q| on the host (it overlaps the copies just queued), unless given
  c->norm_q = norm_q >= 0.0 ? norm_q : fc3dgpu_norm_q_host(q, 3LL * nc);
  if (c->nscenes > 0) {
    c->scene_normq_h.assign(c->nscenes, 0.0);
    for (int g = 0; g < c->nscenes; g++) {
      double t = 0.0;
      for (long long i = 3LL * c->scene_off_h[g]; i < 3LL * c->scene_off_h[g + 1]; i++) t += q[i] * q[i];
      c->scene_normq_h[g] = sqrt(t);
    }
    CK(ensure(&c->snormq, &c->snormq_cap, (size_t)c->nscenes));
    CK(cudaMemcpyAsync(c->snormq, c->scene_normq_h.data(), sizeof(double) * c->nscenes, cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  c->have_q = true;
  return 0;
}

extern "C" int fc3dgpu_ctx_set_r(fc3dgpu_ctx* c, const double* r) {
  using namespace fc3dgpu;
  if (!c || !c->have_W || !r) {
    fc3dgpu_set_error("fc3dgpu_ctx_set_r: W not set or null input");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  CK(cudaSetDevice(c->device));
  const int nc = c->nc;
  CK(ensure(&c->ro, &c->ro_cap, (size_t)nc * 3));
  CK(cudaMemcpyAsync(c->ro, r, sizeof(double) * 3 * nc, cudaMemcpyHostToDevice, c->stream));
  k_set_r<<<grid1d(nc), 256, 0, c->stream>>>(nc, c->iperm, c->ro, c->r64, c->r32, c->rpli64, c->rpli32);
  CK(cudaGetLastError());
  c->launches++;
  c->have_r = true;
  return 0;
}

// Reset the iterate on the device: r = 0 and the PLI steps to 1, as a solve
// from a zero warm start after fc3dgpu_ctx_set_r(zeros) would have them.
__global__ void k_zero_r(int npad, double* __restrict__ r64, float* __restrict__ r32, double* __restrict__ rpli64,
                         float* __restrict__ rpli32) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p <= npad; p += gridDim.x * blockDim.x) {
    for (int a = 0; a < 4; a++) {
      r64[4 * (size_t)p + a] = 0.0;
      r32[4 * (size_t)p + a] = 0.0f;
    }
    if (p < npad) {
      rpli64[p] = 1.0;
      rpli32[p] = 1.0f;
    }
  }
}

// Synchronisation between the colours of a sweep (one lane per contact):
// 1 (default) each block waits only for the blocks it shares W blocks with,
// 0 every block waits for all.  Returns the previous setting.
extern "C" int fc3dgpu_ctx_sync(fc3dgpu_ctx* c, int neighbourhood) {
  if (!c) return -1;
  const int old = c->nbr_sync;
  c->nbr_sync = neighbourhood ? 1 : 0;
  return old;
}

// Bulk-copy staging of slab ranges in the FP32 sweeps: on (1, default) or
// off (0).  Returns the previous setting.
extern "C" int fc3dgpu_ctx_staging(fc3dgpu_ctx* c, int on) {
  if (!c) return -1;
  const int old = c->staging;
  c->staging = on ? 1 : 0;
  return old;
}

// Slab-dataflow FP32 sweep (no barriers between colours): on (1, default)
// or off (0, the coloured persistent kernel).  Returns the previous setting.
extern "C" int fc3dgpu_ctx_flow(fc3dgpu_ctx* c, int on) {
  if (!c) return -1;
  const int old = c->flow_on;
  c->flow_on = on ? 1 : 0;
  return old;
}

extern "C" int fc3dgpu_ctx_flow_warps(fc3dgpu_ctx* c, int nw) {
  if (!c) return -1;
  if (nw != 0 && nw != 8 && nw != 10 && nw != 12) {
    fc3dgpu_set_error("fc3dgpu_ctx_flow_warps: 8, 10 or 12 warps per block (0: default)");
    return NUMERICS_ERR_INVALID_OPTION;
  }
  const int old = c->flow_want;
  c->flow_want = nw;
  if (c->flow_state == 1) {
    if (cudaSetDevice(c->device) != cudaSuccess) return NUMERICS_ERR_UNKNOWN;
    const int got = fc3dgpu::flow_warps(c->flow_maxslot, nw);
    if (got > 0) c->flow_nw = got;
  }
  return old;
}

// Polls before a barrier, slab-counter or bulk-copy wait of the sweep
// kernels gives up (0: the default 2^22); a wait that gives up sets
// FC3DGPU_STATUS_BARRIER_TIMEOUT and the solve returns an error.  Returns
// the previous setting.
extern "C" unsigned long long fc3dgpu_ctx_spin_limit(fc3dgpu_ctx* c, unsigned long long polls) {
  if (!c) return 0;
  const unsigned long long old = c->spin_limit;
  c->spin_limit = polls;
  return old;
}

extern "C" int fc3dgpu_ctx_zero_r(fc3dgpu_ctx* c) {
  if (!c || !c->have_W) {
    fc3dgpu_set_error("fc3dgpu_ctx_zero_r: no problem");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  CK(cudaSetDevice(c->device));
  k_zero_r<<<grid1d(c->npad + 1), 256, 0, c->stream>>>(c->npad, c->r64, c->r32, c->rpli64, c->rpli32);
  CK(cudaGetLastError());
  c->launches++;
  c->have_r = true;
  return 0;
}

// Device facts: [0] SMs, [1] L2 bytes, [2] pageable host memory readable
// by kernels, [3] ... through the host page tables, [4] cooperative launch,
// [5] compute capability major*10+minor.  Returns 0 or a negative code.
extern "C" int fc3dgpu_device_info(int device, long long* out6) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    fc3dgpu_set_error("no CUDA device %d", device);
    return NUMERICS_ERR_NOT_IMPLEMENTED;
  }
  int v[6] = {0, 0, 0, 0, 0, 0}, ma = 0, mi = 0;
  cudaDeviceGetAttribute(&v[0], cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&v[1], cudaDevAttrL2CacheSize, device);
  cudaDeviceGetAttribute(&v[2], cudaDevAttrPageableMemoryAccess, device);
  cudaDeviceGetAttribute(&v[3], cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
  cudaDeviceGetAttribute(&v[4], cudaDevAttrCooperativeLaunch, device);
  cudaDeviceGetAttribute(&ma, cudaDevAttrComputeCapabilityMajor, device);
  cudaDeviceGetAttribute(&mi, cudaDevAttrComputeCapabilityMinor, device);
  v[5] = ma * 10 + mi;
  for (int i = 0; i < 6; i++) out6[i] = v[i];
  return 0;
}

extern "C" void* fc3dgpu_ctx_stream(fc3dgpu_ctx* c) { return c ? (void*)c->stream : nullptr; }

extern "C" unsigned long long fc3dgpu_ctx_launches(fc3dgpu_ctx* c) { return c ? c->launches : 0; }

extern "C" int fc3dgpu_ctx_get_r_u(fc3dgpu_ctx* c, double* r, double* u) {
  using namespace fc3dgpu;
  if (!c || !c->have_W) {
    fc3dgpu_set_error("fc3dgpu_ctx_get_r_u: no problem");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  CK(cudaSetDevice(c->device));
  const int nc = c->nc;
  CK(ensure(&c->ro, &c->ro_cap, (size_t)nc * 3));
  CK(ensure(&c->uo, &c->uo_cap, (size_t)nc * 3));
  k_get_r_u<<<grid1d(nc), 256, 0, c->stream>>>(nc, c->iperm, c->r64, c->u64, c->ro, c->uo);
  CK(cudaGetLastError());
  c->launches++;
  if (r) CK(cudaMemcpyAsync(r, c->ro, sizeof(double) * 3 * nc, cudaMemcpyDeviceToHost, c->stream));
  if (u) CK(cudaMemcpyAsync(u, c->uo, sizeof(double) * 3 * nc, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

template <typename Real>
static void fill_args(fc3dgpu_ctx* c, fc3dgpu::SweepArgs<Real>& a, const Real* W, const Real* D, const Real* q,
                      const Real* mu, const Real* rho, Real* r, Real* rpli) {
  a.ncol = c->ncol;
  a.nslab = c->nslab;
  a.npad = c->npad;
  for (int k = 0; k <= FC3D_MAX_COLOURS; k++) a.sptr[k] = c->sptr[k];
  a.slab_nslot = c->slab_nslot;
  a.slab_off = c->slab_off;
  a.perm = c->perm;
  a.dpos = c->dpos;
  a.W = W;
  a.col = c->col;
  a.D = D;
  a.q = q;
  a.mu = mu;
  a.rho = rho;
  a.r = r;
  a.rpli = rpli;
  a.u = c->u64;
  a.partials = c->partials;
  a.barrier = c->barrier;
  a.status = c->status;
  a.trace = c->trace;
  a.trace_cap = (int)c->trace_cap;
  a.trace_base = 0;
  a.norm_q = c->norm_q;
  a.spin_limit = c->spin_limit ? c->spin_limit : 1ULL << 22;
  a.counters = c->counters_on ? c->counters : nullptr;
  a.timeline = c->timeline_sweep > 0 ? c->timeline : nullptr;
  a.timeline_sweep = c->timeline_sweep;
  a.stage_w_bytes = a.stage_c_bytes = a.stage_q_bytes = a.stage_d_bytes = 0;
  for (int k = 0; k < FC3D_MAX_COLOURS; k++) a.ccount[k] = c->ccount[k];
  a.out = c->out;
  a.nbr_ptr = nullptr;
  a.nbr = nullptr;
  a.nbr_grid = 0;
  a.local_mode = 0;
  a.relax = 0;
  a.filter = 0;
  a.omega = 1.0;
}

// Neighbour lists of every block for a sweep over `grid` blocks (one lane
// per contact): built once per layout and grid size.
template <typename Real>
static int attach_nbr(fc3dgpu_ctx* c, fc3dgpu::SweepArgs<Real>& a, int grid) {
  using namespace fc3dgpu;
  if (!c->nbr_sync || grid <= 0 || c->nscenes > 0 || c->ncol < 2) return 0;
  fc3dgpu_ctx::Nbr* hit = nullptr;
  for (auto& n : c->nbrc)
    if (n.grid == grid) hit = &n;
  if (!hit) {
    hit = &c->nbrc[c->nbr_next];
    c->nbr_next ^= 1;
    hit->grid = 0;
    const int words = (grid + 31) / 32;
    cudaStream_t s = c->stream;
    CK(ensure(&c->nbrmask, &c->nbrmask_cap, (size_t)grid * words));
    CK(cudaMemsetAsync(c->nbrmask, 0, sizeof(unsigned) * grid * words, s));
    ColourBounds cb;
    for (int k = 0; k <= FC3D_MAX_COLOURS; k++) cb.sptr[k] = c->sptr[k];
    k_block_adjacency<<<grid1d((long long)c->nslab * FC3D_SLAB), 256, 0, s>>>(
        c->nslab, c->npad, cb, c->ncol, grid, words, c->perm, c->slab_nslot, c->slab_off, c->col, c->nbrmask);
    CK(cudaGetLastError());
    c->launches++;
    std::vector<unsigned> mask((size_t)grid * words);
    CK(cudaMemcpyAsync(mask.data(), c->nbrmask, sizeof(unsigned) * mask.size(), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    std::vector<int> ptr(grid + 1, 0), list;
    for (int b = 0; b < grid; b++) {
      for (int b2 = 0; b2 < grid; b2++)
        if (mask[(size_t)b * words + b2 / 32] & (1u << (b2 % 32))) list.push_back(b2);
      ptr[b + 1] = (int)list.size();
    }
    if (hit->ptr) cudaFree(hit->ptr);
    if (hit->list) cudaFree(hit->list);
    hit->ptr = hit->list = nullptr;
    CK(cudaMalloc(&hit->ptr, sizeof(int) * (grid + 1)));
    CK(cudaMalloc(&hit->list, sizeof(int) * (list.empty() ? 1 : list.size())));
    CK(cudaMemcpyAsync(hit->ptr, ptr.data(), sizeof(int) * (grid + 1), cudaMemcpyHostToDevice, s));
    if (!list.empty())
      CK(cudaMemcpyAsync(hit->list, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    hit->grid = grid;
  }
  a.nbr_ptr = hit->ptr;
  a.nbr = hit->list;
  a.nbr_grid = grid;
  return 0;
}

// Staging buffer sizes (bytes of W, col, q) for the largest slab range one
// of `grid` blocks takes in any colour; 0 when staging cannot be used
// (a range longer than one pass, or more shared memory than a block has).
template <typename Real>
static size_t staging_sizes(fc3dgpu_ctx* c, int grid, unsigned* wb, unsigned* cb, unsigned* qb, unsigned* db) {
  *wb = *cb = *qb = *db = 0;
  if (!c->staging || grid <= 0) return 0;
  size_t mw = 0, mc = 0, mq = 0, md = 0;
  for (int col = 0; col < c->ncol; col++) {
    const int s0 = c->sptr[col], n = c->sptr[col + 1] - s0;
    for (int b = 0; b < grid; b++) {
      const int lo = s0 + (int)((long long)n * b / grid), hi = s0 + (int)((long long)n * (b + 1) / grid);
      if (hi <= lo) continue;
      if (hi - lo > 16) return 0;
      const long long o0 = c->slab_off_h[lo];
      const long long o1 = hi < c->nslab ? c->slab_off_h[hi] : c->slab_off_h[hi - 1] + c->slab_nslot_h[hi - 1];
      const size_t slots = (size_t)(o1 - o0);
      mw = std::max(mw, slots * 9 * FC3D_SLAB * sizeof(Real));
      mc = std::max(mc, slots * FC3D_SLAB * sizeof(int));
      mq = std::max(mq, (size_t)(hi - lo) * 3 * FC3D_SLAB * sizeof(Real));
      md = std::max(md, (size_t)(hi - lo) * 9 * FC3D_SLAB * sizeof(Real));
    }
  }
  const size_t buffers = (mw + mc + mq + md / 9 * 12 + 15) & ~(size_t)15;
  const size_t tot = buffers + sizeof(fc3dgpu::WorkListS<Real>);
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  // static shared memory of the kernel: the direct-load work list and a few
  // reduction arrays
  const size_t static_smem = sizeof(fc3dgpu::WorkList<Real>) + 2048;
  if (tot + static_smem > (size_t)optin) return 0;
  *wb = (unsigned)mw;
  *cb = (unsigned)mc;
  *qb = (unsigned)mq;
  *db = (unsigned)md;
  return tot;
}

// Column-slab lists of the dataflow sweep for the current layout; leaves
// c->flow_state 1 when the sweep applies, -1 when not (slabs longer than
// FC3D_FLOW_MAXSLOT or than the per-warp buffers allow).
static int prepare_flow(fc3dgpu_ctx* c) {
  using namespace fc3dgpu;
  if (c->flow_state != 0) return 0;
  c->flow_state = -1;
  if (c->nscenes > 0 || c->ncol < 2 || c->nslab <= 0) return 0;
  int maxslot = 0;
  for (int s = 0; s < c->nslab; s++) maxslot = std::max(maxslot, c->slab_nslot_h[s]);
  if (maxslot > FC3D_FLOW_MAXSLOT) return 0;
  const int nw = flow_warps(maxslot, c->flow_want);
  if (nw == 0) return 0;
  cudaStream_t s = c->stream;
  const int nslab = c->nslab;
  CK(ensure(&c->flow_dptr, &c->flow_dptr_cap, (size_t)nslab + 1));
  CK(ensure(&c->flow_done, &c->flow_done_cap, (size_t)nslab));
  CK(ensure(&c->flow_sptr, &c->flow_sptr_cap, FC3D_MAX_COLOURS + 1));
  CK(ensure(&c->flow_part, &c->flow_part_cap, 1024 * 8));
  CK(cudaMemcpyAsync(c->flow_sptr, c->sptr, sizeof(int) * (FC3D_MAX_COLOURS + 1), cudaMemcpyHostToDevice, s));
  // column-slab counts, their prefix sum on the host, then the lists
  CK(build_flow_deps(nslab, c->npad, c->ncol, c->flow_sptr, c->perm, c->slab_nslot, c->slab_off, c->col, nullptr,
                     c->flow_dptr, nullptr, s));
  std::vector<int> ptr((size_t)nslab + 1, 0);
  CK(cudaMemcpyAsync(ptr.data() + 1, c->flow_dptr, sizeof(int) * nslab, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int k = 0; k < nslab; k++) ptr[k + 1] += ptr[k];
  CK(ensure(&c->flow_dep, &c->flow_dep_cap, (size_t)std::max(ptr[nslab], 1)));
  CK(cudaMemcpyAsync(c->flow_dptr, ptr.data(), sizeof(int) * (nslab + 1), cudaMemcpyHostToDevice, s));
  CK(build_flow_deps(nslab, c->npad, c->ncol, c->flow_sptr, c->perm, c->slab_nslot, c->slab_off, c->col,
                     c->flow_dptr, nullptr, c->flow_dep, s));
  std::vector<int> cols((size_t)std::max(ptr[nslab], 1));
  CK(cudaMemcpyAsync(cols.data(), c->flow_dep, sizeof(int) * ptr[nslab], cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  // Symmetric lists: the slabs s takes columns from and the slabs that take
  // columns from s (the same sets when W's block pattern is symmetric, as a
  // Delassus operator's is).  A finished slab signals every slab of its
  // list, and a slab of a later colour that s reads must wait for s even
  // when it does not read s.
  std::vector<int> rptr((size_t)nslab + 1, 0);
  for (int k = 0; k < ptr[nslab]; k++) rptr[(cols[k] & 0x7fffffff) + 1]++;
  for (int k = 0; k < nslab; k++) rptr[k + 1] += rptr[k];
  std::vector<int> rev((size_t)std::max(rptr[nslab], 1)), fill(rptr.begin(), rptr.end() - 1);
  for (int t = 0; t < nslab; t++)  // ascending t: each reverse list comes out sorted
    for (int k = ptr[t]; k < ptr[t + 1]; k++) rev[fill[cols[k] & 0x7fffffff]++] = t;
  auto colour_of = [&](int sl) { return (int)(std::upper_bound(c->sptr, c->sptr + c->ncol + 1, sl) - c->sptr) - 1; };
  std::vector<int> sym, sptr_sym((size_t)nslab + 1, 0);
  std::vector<int2> need((size_t)nslab);
  sym.reserve((size_t)ptr[nslab] + 16);
  for (int t = 0; t < nslab; t++) {
    const int ct = colour_of(t);
    int a = ptr[t], b = rptr[t], nhi = 0;
    const size_t start = sym.size();
    while (a < ptr[t + 1] || b < rptr[t + 1]) {
      const int x = a < ptr[t + 1] ? (cols[a] & 0x7fffffff) : INT_MAX;
      const int y = b < rptr[t + 1] ? rev[b] : INT_MAX;
      const int d = std::min(x, y);
      if (x == d) a++;
      if (y == d) b++;
      const bool hi = colour_of(d) > ct;
      nhi += hi;
      sym.push_back(hi ? (int)((unsigned)d | 0x80000000u) : d);
    }
    sptr_sym[t + 1] = (int)sym.size();
    need[t] = make_int2((int)(sym.size() - start), nhi);
  }
  CK(ensure(&c->flow_dep, &c->flow_dep_cap, std::max(sym.size(), (size_t)1)));
  CK(ensure(&c->flow_need, &c->flow_need_cap, (size_t)nslab));
  CK(cudaMemcpyAsync(c->flow_dptr, sptr_sym.data(), sizeof(int) * (nslab + 1), cudaMemcpyHostToDevice, s));
  if (!sym.empty()) CK(cudaMemcpyAsync(c->flow_dep, sym.data(), sizeof(int) * sym.size(), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->flow_need, need.data(), sizeof(int2) * nslab, cudaMemcpyHostToDevice, s));
  // offsets of the per-slab records (filled before each solve's FP32 sweeps)
  std::vector<long long> roff((size_t)nslab + 1, 0);
  for (int t = 0; t < nslab; t++) roff[t + 1] = roff[t] + flow_rec_floats(c->slab_nslot_h[t]);
  CK(ensure(&c->flow_rec_off, &c->flow_rec_off_cap, (size_t)nslab + 1));
  CK(ensure(&c->flow_rec, &c->flow_rec_cap, (size_t)std::max(roff[nslab], 1LL)));
  CK(cudaMemcpyAsync(c->flow_rec_off, roff.data(), sizeof(long long) * (nslab + 1), cudaMemcpyHostToDevice, s));
  CK(cudaStreamSynchronize(s));
  c->launches += 2;
  c->flow_nw = nw;
  c->flow_maxslot = maxslot;
  c->flow_state = 1;
  return 0;
}

// Measuring autotuner.  At the first solve of a layout with automatic lanes
// it times FP32 sweeps of the candidate variants, each as one warm-up solve
// and one measured solve (device time from CUDA events) from the current
// reaction, which is restored afterwards, and keeps the fastest for the
// layout (a new structure tunes again).  Mode 1 (the default) weighs only
// variants that give the same iterates bit for bit: the dataflow sweep with
// 8, 10 or 12 warps a block (each warp stages its own slab, so this is the
// staging depth of an SM) and the coloured kernel with one lane per contact
// (bulk-copy staged); FP64 sweeps keep one lane per contact (the oracle's
// iterates).  Mode 2 adds the coloured kernel with 2, 4 and 8 lanes per
// contact in both precisions (a row's product split over lanes: other sums,
// so the choice shows in the last bits); mode 0 uses the defaults unmeasured.
// On the 60x60x30 lattice mode 1 costs about 3 ms once per structure.
static int solve_impl(fc3dgpu_ctx* c, const fc3dgpu_params* p, fc3dgpu_stats* st);

static float tune_one(fc3dgpu_ctx* c, const fc3dgpu_params& base, int precision, int lanes, int sweeps) {
  fc3dgpu_params q = base;
  q.precision = precision;
  q.lanes = lanes;
  q.tol = 1e-300;
  q.switch_tol = 0.0;
  q.stall_window = 0;
  q.fp32_only = precision == 0 ? 1 : 0;
  fc3dgpu_stats S;
  q.max_iter = 2;
  if (solve_impl(c, &q, &S) != 0) return INFINITY;
  q.max_iter = sweeps;
  if (solve_impl(c, &q, &S) != 0) return INFINITY;
  const double ms = precision == 0 ? S.ms_fp32 : S.ms_fp64;
  const int n = precision == 0 ? S.sweeps32 : S.sweeps64;
  return n > 0 ? (float)(ms / n) : INFINITY;
}

static int autotune(fc3dgpu_ctx* c, const fc3dgpu_params* p) {
  using namespace fc3dgpu;
  if (c->tuned) return 0;
  cudaStream_t s = c->stream;
  const size_t nr = ((size_t)c->npad + 1) * 4;
  CK(ensure(&c->tune_r64, &c->tune_r64_cap, nr));
  CK(ensure(&c->tune_rpli64, &c->tune_rpli64_cap, (size_t)c->npad));
  CK(ensure(&c->tune_rpli32, &c->tune_rpli32_cap, (size_t)c->npad));
  CK(cudaMemcpyAsync(c->tune_r64, c->r64, sizeof(double) * nr, cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(c->tune_rpli64, c->rpli64, sizeof(double) * c->npad, cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(c->tune_rpli32, c->rpli32, sizeof(float) * c->npad, cudaMemcpyDeviceToDevice, s));
  const int flow_on = c->flow_on, want = c->flow_want;
  unsigned long long* tl = c->timeline;
  const int tls = c->timeline_sweep, cnt = c->counters_on;
  c->timeline_sweep = 0;
  c->counters_on = 0;
  const int sw32 = 6, sw64 = 3;
  const bool all = c->tune_mode >= 2;
  float best32 = INFINITY, best64 = INFINITY;
  int k = 0;
  c->tune_flow = 0;
  c->tune_nw = 0;
  c->tune_lanes32 = 1;
  c->tune_lanes64 = 1;
  // the dataflow sweep at 8, 10, 12 warps a block
  c->flow_on = 1;
  if (int rc = prepare_flow(c)) return rc;
  const bool flow_ok = c->flow_state == 1;
  const int nws[3] = {8, 10, 12};
  for (int i = 0; i < 3; i++, k++) {
    c->tune_ms32[k] = INFINITY;
    if (!flow_ok) continue;
    const int got = flow_warps(c->flow_maxslot, nws[i]);
    if (got != nws[i]) continue;
    c->flow_nw = got;
    const float ms = tune_one(c, *p, 0, 1, sw32);
    c->tune_ms32[k] = ms;
    if (ms < best32) {
      best32 = ms;
      c->tune_flow = 1;
      c->tune_nw = got;
      c->tune_lanes32 = 1;
    }
  }
  // the coloured kernel at 1 (and, in mode 2, 2, 4, 8) lanes per contact
  c->flow_on = 0;
  const int ls[4] = {1, 2, 4, 8};
  for (int i = 0; i < 4; i++, k++) {
    c->tune_ms32[k] = INFINITY;
    if (i > 0 && !all) continue;
    const float ms = tune_one(c, *p, 0, ls[i], sw32);
    c->tune_ms32[k] = ms;
    if (ms < best32) {
      best32 = ms;
      c->tune_flow = 0;
      c->tune_lanes32 = ls[i];
    }
  }
  for (int i = 0; i < 4; i++) {
    c->tune_ms64[i] = INFINITY;
    if (!all) continue;
    const float ms = tune_one(c, *p, 1, ls[i], sw64);
    c->tune_ms64[i] = ms;
    if (ms < best64) {
      best64 = ms;
      c->tune_lanes64 = ls[i];
    }
  }
  if (!all) best64 = 0.f;  // one lane per contact, unmeasured
  c->flow_on = flow_on;
  c->flow_want = want;
  if (c->flow_state == 1) c->flow_nw = c->tune_flow ? c->tune_nw : flow_warps(c->flow_maxslot, want);
  c->timeline = tl;
  c->timeline_sweep = tls;
  c->counters_on = cnt;
  CK(cudaMemcpyAsync(c->r64, c->tune_r64, sizeof(double) * nr, cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(c->rpli64, c->tune_rpli64, sizeof(double) * c->npad, cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(c->rpli32, c->tune_rpli32, sizeof(float) * c->npad, cudaMemcpyDeviceToDevice, s));
  CK(cudaStreamSynchronize(s));
  if (!(best32 < INFINITY) || !(best64 < INFINITY)) {
    fc3dgpu_set_error("autotuner: no sweep variant ran");
    return NUMERICS_ERR_UNKNOWN;
  }
  c->tuned = 1;
  return 0;
}

extern "C" int fc3dgpu_ctx_autotune(fc3dgpu_ctx* c, int mode) {
  if (!c) return -1;
  if (mode < 0 || mode > 2) {
    fc3dgpu_set_error("fc3dgpu_ctx_autotune: mode 0, 1 or 2");
    return NUMERICS_ERR_INVALID_OPTION;
  }
  const int old = c->tune_mode;
  if (mode != old) c->tuned = 0;
  c->tune_mode = mode;
  return old;
}

extern "C" int fc3dgpu_ctx_tuning(fc3dgpu_ctx* c, int* choice4, float* ms11) {
  if (!c) return NUMERICS_ERR_NULL_POINTER;
  if (!c->tuned) return 1;
  if (choice4) {
    choice4[0] = c->tune_flow;
    choice4[1] = c->tune_flow ? c->tune_nw : 0;
    choice4[2] = c->tune_lanes32;
    choice4[3] = c->tune_lanes64;
  }
  if (ms11) {
    for (int i = 0; i < 7; i++) ms11[i] = c->tune_ms32[i];
    for (int i = 0; i < 4; i++) ms11[7 + i] = c->tune_ms64[i];
  }
  return 0;
}

extern "C" int fc3dgpu_ctx_solve(fc3dgpu_ctx* c, const fc3dgpu_params* p, fc3dgpu_stats* st) {
  if (!c || !p || !c->have_W || !c->have_q || !c->have_r) {
    fc3dgpu_set_error("fc3dgpu_ctx_solve: problem, q/mu or r not set");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (p->lanes <= 0 && !c->tuned && c->tune_mode > 0 && c->nscenes == 0) {
    if (cudaSetDevice(c->device) != cudaSuccess) {
      fc3dgpu_set_error("fc3dgpu_ctx_solve: cudaSetDevice(%d) failed", c->device);
      return NUMERICS_ERR_UNKNOWN;
    }
    if (int rc = autotune(c, p)) return rc;
  }
  return solve_impl(c, p, st);
}

static int solve_impl(fc3dgpu_ctx* c, const fc3dgpu_params* p, fc3dgpu_stats* st) {
  using namespace fc3dgpu;
  if (!c || !p || !c->have_W || !c->have_q || !c->have_r) {
    fc3dgpu_set_error("fc3dgpu_ctx_solve: problem, q/mu or r not set");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  CK(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  fc3dgpu_stats S;
  memset(&S, 0, sizeof(S));
  // automatic lanes: the autotuner's choices for this layout (without it,
  // one lane per contact and the dataflow sweep where it applies)
  const bool tuned = p->lanes <= 0 && c->tuned;
  const int lanes64 = p->lanes > 0 ? p->lanes : (tuned ? c->tune_lanes64 : 1);
  const int lanes = p->lanes > 0 ? p->lanes : (tuned ? c->tune_lanes32 : 1);
  const bool use_flow = c->flow_on && (!tuned || c->tune_flow);
  const bool mixed = p->precision == 0 || p->precision == 2, fast64 = p->precision >= 2;
  if (p->precision < 0 || p->precision > 3) {
    fc3dgpu_set_error("precision must be 0, 1, 2 or 3 (got %d)", p->precision);
    return NUMERICS_ERR_INVALID_OPTION;
  }
  if (p->local_mode32 != 0 && p->local_mode32 != 1) {
    fc3dgpu_set_error("local_mode32 must be 0 or 1 (got %d)", p->local_mode32);
    return NUMERICS_ERR_INVALID_OPTION;
  }
  if (lanes64 != 1 && lanes64 != 2 && lanes64 != 4 && lanes64 != 8) {
    fc3dgpu_set_error("lanes per contact must be 1, 2, 4 or 8 (got %d)", lanes64);
    return NUMERICS_ERR_INVALID_OPTION;
  }
  S.lanes = lanes;
  S.colours = c->ncol;
  const double s32 = 4.0, s64 = 8.0;
  S.bytes_sweep32 = (double)c->nnzb * (9 * s32 + 4) + (double)c->nc * (3 * s32 + s32 + 3 * s32 + 3 * s32);
  S.bytes_sweep64 = (double)c->nnzb * (9 * s64 + 4) + (double)c->nc * (3 * s64 + s64 + 3 * s64 + 3 * s64);
  CK(cudaMemsetAsync(c->status, 0, sizeof(int), s));
  CK(cudaEventRecord(c->ev[0], s));
  int sweeps32 = 0, grid = 0;
  bool converged32 = false;
  double out[8];
  if (mixed && p->max_iter > 0) {
    SweepArgs<float> a;
    fill_args<float>(c, a, c->W32, c->D32, c->q32, c->mu32, c->rho32, c->r32, c->rpli32);
    a.max_sweeps = p->max_iter;
    a.mode = 0;
    a.user_tol = p->tol;
    a.local_tol = p->local_tol32;
    a.switch_tol = p->switch_tol;
    a.stall_window = p->stall_window;
    a.newton_max = p->newton_max;
    a.pli_max = p->pli_max;
    a.ls_max = p->ls_max;
    a.local_mode = p->local_mode32;
    size_t smem = 0;
    if (lanes == 1) {
      const int g1 = sweep_grid_f32(1);
      smem = staging_sizes<float>(c, g1, &a.stage_w_bytes, &a.stage_c_bytes, &a.stage_q_bytes, &a.stage_d_bytes);
    }
    // the FP32 sweeps start from the context's reaction (the FP64 iterate of
    // a previous solve, a warm start, or what fc3dgpu_ctx_set_r gave)
    k_r64_to_r32<<<grid1d(c->npad), 256, 0, s>>>(c->npad, c->r64, c->r32);
    CK(cudaGetLastError());
    c->launches++;
    bool flow = lanes == 1 && use_flow && !a.counters;
    if (flow) {
      if (int rc = prepare_flow(c)) return rc;
      flow = c->flow_state == 1;
    }
    if (lanes == 1 && !flow)
      if (int rc = attach_nbr<float>(c, a, sweep_grid_f32(1))) return rc;
    CK(cudaMemsetAsync(c->barrier, 0, FC3D_BARRIER_WORDS * sizeof(unsigned), s));
    if (flow) {
      // the per-slab timeline fits the buffer up to this many slabs
      if (c->nslab > FC3D_MAX_COLOURS * 1024) a.timeline = nullptr;
      FlowArgs f;
      f.dptr = c->flow_dptr;
      f.dep = c->flow_dep;
      f.done = c->flow_done;
      f.need = c->flow_need;
      f.part = c->flow_part;
      f.maxslot = c->flow_maxslot;
      f.buf_bytes = flow_buf_bytes(c->flow_maxslot);
      f.rec = c->flow_rec;
      f.rec_off = c->flow_rec_off;
      CK(cudaMemsetAsync(c->flow_done, 0, sizeof(unsigned) * c->nslab, s));
      CK(pack_flow_records(c->nslab, c->slab_off, c->slab_nslot, c->W32, c->col, c->q32, c->D32, c->mu32, c->rho32,
                           c->flow_rec_off, c->flow_rec, s));
      c->launches++;
      CK(launch_flow_f32(a, f, c->flow_nw, s, &grid));
    } else {
      CK(launch_sweep_f32(a, lanes, 0, smem, s, &grid));
    }
    c->launches++;
    CK(cudaMemcpyAsync(out, c->out, sizeof(double) * 6, cudaMemcpyDeviceToHost, s));
    CK(cudaEventRecord(c->ev[1], s));
    CK(cudaStreamSynchronize(s));
    sweeps32 = (int)out[0];
    S.incr_error = out[1];
    converged32 = out[3] == 0.0;
    k_r32_to_r64<<<grid1d(c->npad), 256, 0, s>>>(c->npad, c->r32, c->rpli32, c->r64, c->rpli64);
    CK(cudaGetLastError());
    c->launches++;
  } else {
    CK(cudaEventRecord(c->ev[1], s));
  }
  {
    SweepArgs<double> a;
    fill_args<double>(c, a, c->W64, c->D64, c->q64, c->mu64, c->rho64, c->r64, c->rpli64);
    int budget = p->max_iter - sweeps32;
    if (budget < 0 || p->fp32_only) budget = 0;
    a.max_sweeps = budget;
    a.mode = 1;
    a.user_tol = p->tol;
    a.local_tol = p->local_tol;
    a.switch_tol = 0.0;
    a.stall_window = 0;
    a.trace_base = sweeps32;
    a.relax = p->relax;
    a.omega = p->omega;
    a.filter = p->filter;
    a.newton_max = p->newton_max;
    a.pli_max = p->pli_max;
    a.ls_max = p->ls_max;
    int g64 = 0;
    if (lanes64 == 1)
      if (int rc = attach_nbr<double>(c, a, sweep_grid_f64(1))) return rc;
    // the exact FP64 kernels, or those with the fast one-contact arithmetic
    // (same grid: same occupancy)
    auto launch64 = [&](const SweepArgs<double>& x) {
      return fast64 ? fc3dgpu_launch_sweep_f64_fast(&x, lanes64, 0, s, &g64)
                    : launch_sweep_f64(x, lanes64, 0, 0, s, &g64);
    };
    if (converged32 && budget > 0) {
      // the FP32 iterate met the tolerance in FP32 arithmetic: check it in
      // FP64 before any FP64 sweep
      a.max_sweeps = 0;
      CK(cudaMemsetAsync(c->barrier, 0, FC3D_BARRIER_WORDS * sizeof(unsigned), s));
      CK(launch64(a));
      c->launches++;
      CK(cudaMemcpyAsync(out, c->out, sizeof(double) * 6, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      a.max_sweeps = out[3] == 0.0 ? 0 : budget;
    }
    if (!(converged32 && a.max_sweeps == 0)) {
      CK(cudaMemsetAsync(c->barrier, 0, FC3D_BARRIER_WORDS * sizeof(unsigned), s));
      CK(launch64(a));
      c->launches++;
      CK(cudaMemcpyAsync(out, c->out, sizeof(double) * 6, cudaMemcpyDeviceToHost, s));
    }
    if (!grid) grid = g64;
  }
  CK(cudaEventRecord(c->ev[2], s));
  int status = 0;
  CK(cudaMemcpyAsync(&status, c->status, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  float ms1 = 0, ms2 = 0;
  cudaEventElapsedTime(&ms1, c->ev[0], c->ev[1]);
  cudaEventElapsedTime(&ms2, c->ev[1], c->ev[2]);
  S.sweeps32 = sweeps32;
  S.sweeps64 = (int)out[0];
  if (S.sweeps64 > 0 || !mixed) S.incr_error = out[1];
  S.error = out[2];
  S.info = (int)out[3];
  if (p->fp32_only && sweeps32 >= p->max_iter && S.info > 0) S.info = NUMERICS_ERR_MAX_ITER;
  if (!p->fp32_only && S.sweeps32 + S.sweeps64 >= p->max_iter && S.info > 0) S.info = NUMERICS_ERR_MAX_ITER;
  S.ms_fp32 = ms1;
  S.ms_fp64 = ms2;
  S.ms_total = (double)ms1 + (double)ms2;
  S.grid = grid;
  S.status = status;
  c->trace_len = S.sweeps32 + S.sweeps64;
  if (st) *st = S;
  if (status) {
    fc3dgpu_set_error("device status %d (%s)", status,
                      (status & FC3DGPU_STATUS_BARRIER_TIMEOUT) ? "a device wait timed out" : "non-finite iterate");
    return NUMERICS_ERR_UNKNOWN;
  }
  return 0;
}

extern "C" int fc3dgpu_ctx_compute_error(fc3dgpu_ctx* c, double* error) {
  using namespace fc3dgpu;
  if (!c || !c->have_W || !c->have_q || !c->have_r) {
    fc3dgpu_set_error("fc3dgpu_ctx_compute_error: problem, q/mu or r not set");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  CK(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  SweepArgs<double> a;
  fill_args<double>(c, a, c->W64, c->D64, c->q64, c->mu64, c->rho64, c->r64, c->rpli64);
  a.max_sweeps = 0;
  a.mode = 1;
  a.user_tol = 1.0;
  a.local_tol = 1e-14;
  a.switch_tol = 0;
  a.stall_window = 0;
  a.newton_max = 100;
  a.pli_max = 100;
  a.ls_max = 10;
  a.trace = nullptr;
  int g = 0;
  double out[8];
  CK(cudaMemsetAsync(c->barrier, 0, FC3D_BARRIER_WORDS * sizeof(unsigned), s));
  CK(cudaMemsetAsync(c->status, 0, sizeof(int), s));
  CK(launch_sweep_f64(a, 1, 0, 0, s, &g));
  CK(cudaMemcpyAsync(out, c->out, sizeof(double) * 6, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (error) *error = out[2];
  return 0;
}

// Work counters of the local solver, accumulated over the solves after
// they are switched on: Newton iterations, PLI iterations, line-search
// evaluations, local solves, largest Newton count of one local solve.
extern "C" int fc3dgpu_ctx_counters(fc3dgpu_ctx* c, int enable, unsigned long long* out8) {
  if (!c) return -1;
  CK(cudaSetDevice(c->device));
  if (out8) {
    CK(cudaMemcpyAsync(out8, c->counters, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  CK(cudaMemsetAsync(c->counters, 0, 8 * sizeof(unsigned long long), c->stream));
  c->counters_on = enable;
  return 0;
}

// Phase timeline of one sweep of the next solves: for colour c and block b,
// out[(c*grid + b)*8 + {0..5}] = globaltimer (ns) at the phase start, at the
// end of the block's work, after its row-product pass (0 when it had no
// slabs), its number of local solves, and (staged sweeps) after the staging
// wait and after the first slab round; entries 6 and 7 are spare (0).
// sweep = 0 switches it off.
extern "C" int fc3dgpu_ctx_timeline(fc3dgpu_ctx* c, int sweep, unsigned long long* out, int cap) {
  if (!c) return -1;
  CK(cudaSetDevice(c->device));
  const size_t need = (size_t)FC3D_MAX_COLOURS * 1024 * FC3D_TL_STRIDE;
  CK(ensure(&c->timeline, &c->timeline_cap, need));
  int n = 0;
  if (out && c->timeline_sweep > 0) {
    n = cap < (int)need ? cap : (int)need;
    CK(cudaMemcpyAsync(out, c->timeline, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  if (sweep > 0) CK(cudaMemsetAsync(c->timeline, 0, sizeof(unsigned long long) * need, c->stream));
  c->timeline_sweep = sweep;
  return n;
}

extern "C" int fc3dgpu_ctx_set_norm_q(fc3dgpu_ctx* c, double norm_q) {
  if (!c) return -1;
  c->norm_q = norm_q;
  return 0;
}

extern "C" int fc3dgpu_ctx_trace(fc3dgpu_ctx* c, double* out, int cap) {
  if (!c) return -1;
  int n = c->trace_len < (int)c->trace_cap ? c->trace_len : (int)c->trace_cap;
  if (n > cap) n = cap;
  if (n > 0) {
    CK(cudaMemcpyAsync(out, c->trace, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return n;
}

extern "C" int fc3dgpu_ctx_colours(fc3dgpu_ctx* c, int32_t* colour) {
  if (!c || !c->have_W) return -1;
  CK(cudaMemcpyAsync(colour, c->colour, sizeof(int) * c->nc, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return c->ncol;
}

extern "C" int fc3dgpu_colour(int nc, const int64_t* rowptr, const int64_t* colidx, int kind, int32_t* colour) {
  if (nc <= 0 || !rowptr || !colidx || !colour) {
    fc3dgpu_set_error("fc3dgpu_colour: invalid argument");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  fc3dgpu_ctx* c = fc3dgpu_ctx_create(dev);
  if (!c) return NUMERICS_ERR_NOT_IMPLEMENTED;
  const long long nnzb = rowptr[nc];
  int rc = validate_bcsr(nc, rowptr, colidx);
  if (rc) {
    fc3dgpu_ctx_destroy(c);
    return rc;
  }
  if (ensure(&c->rowptr, &c->rowptr_cap, (size_t)nc + 1) != cudaSuccess ||
      ensure(&c->colidx, &c->colidx_cap, (size_t)(nnzb ? nnzb : 1)) != cudaSuccess) {
    fc3dgpu_set_error("fc3dgpu_colour: allocation failed");
    rc = NUMERICS_ERR_MEMORY;
  }
  if (!rc) {
    cudaMemcpy(c->rowptr, rowptr, sizeof(long long) * (nc + 1), cudaMemcpyHostToDevice);
    cudaMemcpy(c->colidx, colidx, sizeof(long long) * nnzb, cudaMemcpyHostToDevice);
    rc = colour_device(c, nc, nnzb, kind);
    if (rc >= 0 && cudaMemcpy(colour, c->colour, sizeof(int) * nc, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = NUMERICS_ERR_UNKNOWN;
  }
  fc3dgpu_ctx_destroy(c);
  return rc;
}

// ---------------------------------------------------------------------------
// Batched solve: every problem of a fc3dgpu_ctx_set_W_batch layout in one
// persistent launch per precision, the whole sequence captured once in a
// CUDA graph and replayed while the parameters stay the same.
// ---------------------------------------------------------------------------
static int record_batch(fc3dgpu_ctx* c, const fc3dgpu_params* p) {
  using namespace fc3dgpu;
  cudaStream_t s = c->stream;
  const int ns = c->nscenes;
  int g = 0;
  CK(cudaMemsetAsync(c->squeue, 0, 2 * sizeof(int), s));
  CK(cudaMemsetAsync(c->sout32, 0, sizeof(double) * 8 * ns, s));
  const bool mixed = p->precision == 0 || p->precision == 2;
  if (mixed && p->max_iter > 0) {
    BatchArgs<float> b;
    fill_args<float>(c, b.base, c->W32, c->D32, c->q32, c->mu32, c->rho32, c->r32, c->rpli32);
    b.base.max_sweeps = p->max_iter;
    b.base.mode = 0;
    b.base.user_tol = p->tol;
    b.base.local_tol = p->local_tol32;
    b.base.switch_tol = p->switch_tol;
    b.base.stall_window = p->stall_window;
    b.base.newton_max = p->newton_max;
    b.base.pli_max = p->pli_max;
    b.base.ls_max = p->ls_max;
    b.base.local_mode = p->local_mode32;
    b.base.trace = nullptr;
    b.base.timeline = nullptr;
    b.nscenes = ns;
    b.order = c->sorder;
    b.scene_ncol = c->sncol;
    b.scene_sptr = c->ssptr;
    b.scene_normq = c->snormq;
    b.scene_budget = nullptr;
    b.queue = c->squeue;
    b.scene_out = c->sout32;
    b.scene_out_prev = nullptr;
    CK(launch_batch_f32(b, c->batch_grid32, s, &g));
    k_r32_to_r64<<<grid1d(c->npad), 256, 0, s>>>(c->npad, c->r32, c->rpli32, c->r64, c->rpli64);
  }
  k_batch_budget<<<grid1d(ns), 256, 0, s>>>(ns, c->sout32, p->fp32_only ? 0 : p->max_iter, c->sbudget);
  {
    BatchArgs<double> b;
    fill_args<double>(c, b.base, c->W64, c->D64, c->q64, c->mu64, c->rho64, c->r64, c->rpli64);
    b.base.max_sweeps = p->max_iter;
    b.base.mode = 1;
    b.base.user_tol = p->tol;
    b.base.local_tol = p->local_tol;
    b.base.switch_tol = 0.0;
    b.base.stall_window = 0;
    b.base.newton_max = p->newton_max;
    b.base.pli_max = p->pli_max;
    b.base.ls_max = p->ls_max;
    b.base.trace = nullptr;
    b.base.timeline = nullptr;
    b.nscenes = ns;
    b.order = c->sorder;
    b.scene_ncol = c->sncol;
    b.scene_sptr = c->ssptr;
    b.scene_normq = c->snormq;
    b.scene_budget = c->sbudget;
    b.queue = c->squeue + 1;
    b.scene_out = c->sout64;
    b.scene_out_prev = mixed ? c->sout32 : nullptr;
    if (p->precision >= 2)
      CK(fc3dgpu_launch_batch_f64_fast(&b, c->batch_grid64f, s, &g));
    else
      CK(launch_batch_f64(b, c->batch_grid64, s, &g));
  }
  return 0;
}

extern "C" int fc3dgpu_ctx_solve_batch(fc3dgpu_ctx* c, const fc3dgpu_params* p, int* sweeps32, int* sweeps64,
                                       double* error, int* info, double* ms) {
  using namespace fc3dgpu;
  if (!c || !p || c->nscenes <= 0 || !c->have_q || !c->have_r) {
    fc3dgpu_set_error("fc3dgpu_ctx_solve_batch: no batch layout, q/mu or r");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  CK(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  const int ns = c->nscenes;
  CK(ensure(&c->sbudget, &c->sbudget_cap, (size_t)ns));
  CK(ensure(&c->squeue, &c->squeue_cap, 2));
  CK(ensure(&c->sout32, &c->sout32_cap, (size_t)ns * 8));
  CK(ensure(&c->sout64, &c->sout64_cap, (size_t)ns * 8));
  if (c->batch_graph && memcmp(&c->batch_graph_params, p, sizeof(*p)) != 0) {
    cudaGraphExecDestroy(c->batch_graph);
    c->batch_graph = nullptr;
  }
  if (!c->batch_graph) {
    if (p->precision < 0 || p->precision > 3 || (p->local_mode32 != 0 && p->local_mode32 != 1)) {
      fc3dgpu_set_error("fc3dgpu_ctx_solve_batch: precision must be 0-3 and local_mode32 0 or 1");
      return NUMERICS_ERR_INVALID_OPTION;
    }
    CK(batch_grid_f32(&c->batch_grid32));
    CK(batch_grid_f64(&c->batch_grid64));
    CK(fc3dgpu_batch_grid_f64_fast(&c->batch_grid64f));
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc = record_batch(c, p);
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    CK(e);
    e = cudaGraphInstantiate(&c->batch_graph, graph, 0);
    cudaGraphDestroy(graph);
    CK(e);
    c->batch_graph_params = *p;
  }
  CK(cudaMemsetAsync(c->status, 0, sizeof(int), s));
  CK(cudaEventRecord(c->ev[0], s));
  CK(cudaGraphLaunch(c->batch_graph, s));
  CK(cudaEventRecord(c->ev[1], s));
  c->launches += 4;
  std::vector<double> o32((size_t)ns * 8), o64((size_t)ns * 8);
  int status = 0;
  CK(cudaMemcpyAsync(o32.data(), c->sout32, sizeof(double) * 8 * ns, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(o64.data(), c->sout64, sizeof(double) * 8 * ns, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&status, c->status, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  float t = 0;
  cudaEventElapsedTime(&t, c->ev[0], c->ev[1]);
  if (ms) *ms = t;
  for (int k = 0; k < ns; k++) {
    const int n32 = (int)o32[(size_t)k * 8], n64 = (int)o64[(size_t)k * 8];
    int inf = (int)o64[(size_t)k * 8 + 3];
    if (n32 + n64 >= p->max_iter && inf > 0) inf = NUMERICS_ERR_MAX_ITER;
    if (sweeps32) sweeps32[k] = n32;
    if (sweeps64) sweeps64[k] = n64;
    if (error) error[k] = o64[(size_t)k * 8 + 2];
    if (info) info[k] = inf;
  }
  if (status) {
    fc3dgpu_set_error("device status %d in the batched solve", status);
    return NUMERICS_ERR_UNKNOWN;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Learned warm start (include/fc3dgpu_mlp.h)
// ---------------------------------------------------------------------------
static int features_impl(fc3dgpu_ctx* c, const double* gap) {
  using namespace fc3dgpu;
  cudaStream_t s = c->stream;
  if (ensure(&c->feat, &c->feat_cap, (size_t)c->npad * FC3DGPU_MLP_FEATURES) != cudaSuccess ||
      ensure(&c->gapo, &c->gapo_cap, (size_t)(c->nc ? c->nc : 1)) != cudaSuccess) {
    fc3dgpu_set_error("warm start: allocation failed");
    return NUMERICS_ERR_MEMORY;
  }
  if (gap) CK(cudaMemcpyAsync(c->gapo, gap, sizeof(double) * c->nc, cudaMemcpyHostToDevice, s));
  k_features<<<grid1d(c->npad), 256, 0, s>>>(c->npad, c->perm, c->D64, c->q64, c->mu64, c->r64,
                                              gap ? c->gapo : nullptr, c->feat);
  CK(cudaGetLastError());
  c->launches++;
  return 0;
}

extern "C" int fc3dgpu_ctx_features(fc3dgpu_ctx* c, const double* gap, float* X) {
  using namespace fc3dgpu;
  if (!c || !X) return NUMERICS_ERR_NULL_POINTER;
  if (!c->have_W || !c->have_q || !c->have_r) {
    fc3dgpu_set_error("fc3dgpu_ctx_features: problem, q/mu or r not set");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  CK(cudaSetDevice(c->device));
  if (int rc = features_impl(c, gap)) return rc;
  float* Xd = nullptr;
  CK(cudaMalloc(&Xd, sizeof(float) * FC3DGPU_MLP_FEATURES * (size_t)(c->nc ? c->nc : 1)));
  k_gather_features<<<grid1d((long long)c->nc * FC3DGPU_MLP_FEATURES), 256, 0, c->stream>>>(c->nc, c->iperm,
                                                                                           c->feat, Xd);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(X, Xd, sizeof(float) * FC3DGPU_MLP_FEATURES * (size_t)c->nc, cudaMemcpyDeviceToHost,
                        c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(Xd);
  CK(e);
  c->launches++;
  return 0;
}

extern "C" int fc3dgpu_ctx_warm_start(fc3dgpu_ctx* c, fc3dgpu_mlp* m, const double* gap, double* out3) {
  using namespace fc3dgpu;
  if (!c || !m) return NUMERICS_ERR_NULL_POINTER;
  if (!c->have_W || !c->have_q || !c->have_r) {
    fc3dgpu_set_error("fc3dgpu_ctx_warm_start: problem, q/mu or r not set");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (c->nscenes > 0) {
    fc3dgpu_set_error("fc3dgpu_ctx_warm_start: batched contexts are not supported");
    return NUMERICS_ERR_NOT_IMPLEMENTED;
  }
  CK(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  if (ensure(&c->prop, &c->prop_cap, (size_t)c->npad * 3) != cudaSuccess ||
      ensure(&c->rbak, &c->rbak_cap, (size_t)c->npad * 4) != cudaSuccess) {
    fc3dgpu_set_error("warm start: allocation failed");
    return NUMERICS_ERR_MEMORY;
  }
  double e0 = 0.0, e1 = INFINITY;
  if (int rc = fc3dgpu_ctx_compute_error(c, &e0)) return rc;
  if (int rc = features_impl(c, gap)) return rc;
  if (int rc = fc3dgpu_mlp_infer_stream(m, (size_t)c->npad, c->feat, c->prop, s)) return rc;
  c->launches++;
  // the full step, then half and a quarter of it from the current reaction:
  // the candidate with the smallest fc3d_compute_error, when below e0
  const int residual = fc3dgpu_mlp_residual(m);
  const double alphas[3] = {1.0, 0.5, 0.25};
  double best_alpha = 0.0;
  for (int i = 0; i < 3; i++) {
    k_take_proposal<<<grid1d(c->npad), 256, 0, s>>>(c->npad, c->perm, c->prop, c->mu64, c->r64, c->r32, c->rbak,
                                                     alphas[i], residual, i == 0);
    CK(cudaGetLastError());
    c->launches++;
    double e = 0.0;
    if (int rc = fc3dgpu_ctx_compute_error(c, &e)) return rc;
    if (e < e1) {  // false for a NaN candidate
      e1 = e;
      best_alpha = alphas[i];
    }
  }
  const bool take = e1 < e0;
  if (take && best_alpha != alphas[2]) {
    k_take_proposal<<<grid1d(c->npad), 256, 0, s>>>(c->npad, c->perm, c->prop, c->mu64, c->r64, c->r32, c->rbak,
                                                     best_alpha, residual, 0);
    CK(cudaGetLastError());
    c->launches++;
    CK(cudaStreamSynchronize(s));
  }
  if (!take) {
    k_restore_r<<<grid1d(c->npad), 256, 0, s>>>(c->npad, c->rbak, c->r64, c->r32);
    CK(cudaGetLastError());
    c->launches++;
    CK(cudaStreamSynchronize(s));
  }
  if (out3) {
    out3[0] = e0;
    out3[1] = e1;
    out3[2] = take ? 1.0 : 0.0;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Device assembly of W = H M^-1 H^T and q = H (v + h g) (include/fc3dgpu.h)
// ---------------------------------------------------------------------------
namespace fc3dgpu {

__global__ void k_body_degree(int nc, const int* __restrict__ A, const int* __restrict__ B, int* __restrict__ deg) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    if (A[c] >= 0) atomicAdd(&deg[A[c]], 1);
    atomicAdd(&deg[B[c]], 1);
  }
}

__global__ void k_body_fill(int nc, const int* __restrict__ A, const int* __restrict__ B,
                            const long long* __restrict__ bptr, int* __restrict__ cur, int* __restrict__ blist) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    if (A[c] >= 0) blist[bptr[A[c]] + atomicAdd(&cur[A[c]], 1)] = c;
    blist[bptr[B[c]] + atomicAdd(&cur[B[c]], 1)] = c;
  }
}

// each body's incident contacts in increasing order (lists are short)
__global__ void k_body_sort(int nb, const long long* __restrict__ bptr, int* __restrict__ blist) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
    const long long p0 = bptr[b], p1 = bptr[b + 1];
    for (long long i = p0 + 1; i < p1; i++) {
      const int v = blist[i];
      long long j = i - 1;
      while (j >= p0 && blist[j] > v) {
        blist[j + 1] = blist[j];
        j--;
      }
      blist[j + 1] = v;
    }
  }
}

// Walk the sorted union of the incident lists of the contact's two bodies:
// the columns of its block row, in increasing order.
template <typename F>
__device__ __forceinline__ void row_columns(int c, const int* A, const int* B, const long long* bptr,
                                            const int* blist, F f) {
  const int a = A[c], b = B[c];
  long long i = a >= 0 ? bptr[a] : 0, ie = a >= 0 ? bptr[a + 1] : 0;
  long long j = bptr[b], je = bptr[b + 1];
  int last = -1;
  while (i < ie || j < je) {
    int v;
    if (j >= je || (i < ie && blist[i] <= blist[j]))
      v = blist[i++];
    else
      v = blist[j++];
    if (v != last) {
      f(v);
      last = v;
    }
  }
}

__global__ void k_row_len(int nc, const int* __restrict__ A, const int* __restrict__ B,
                          const long long* __restrict__ bptr, const int* __restrict__ blist, int* __restrict__ len) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    int n = 0;
    row_columns(c, A, B, bptr, blist, [&](int) { n++; });
    len[c] = n;
  }
}

// Contribution of a body b shared by contacts ci and cj to block W_ij
// (column-major): s_i s_j R_i (I/m - [d_i]x [d_j]x / I) R_j^T, with d the
// contact point minus the body centre and s = +1 for body B, -1 for body A;
// [a]x [b]x = b a^T - (a.b) I.  The operation order is that of the scene
// generator, so the blocks are bit-identical to its host assembly.
__device__ __forceinline__ void add_body_block(int ci, int cj, int b, const int* B, const double* frame,
                                               const double* cpt, const double* bpos, double m, double inert,
                                               double W[9]) {
  const double si = (B[ci] == b) ? 1.0 : -1.0, sj = (B[cj] == b) ? 1.0 : -1.0;
  double di[3], dj[3];
  for (int a = 0; a < 3; a++) {
    di[a] = cpt[3 * (size_t)ci + a] - bpos[3 * (size_t)b + a];
    dj[a] = cpt[3 * (size_t)cj + a] - bpos[3 * (size_t)b + a];
  }
  const double ab = di[0] * dj[0] + di[1] * dj[1] + di[2] * dj[2];
  double K[3][3];
  for (int r = 0; r < 3; r++)
    for (int q = 0; q < 3; q++) {
      const double cxx = dj[r] * di[q] - (r == q ? ab : 0.0);
      K[r][q] = (r == q ? 1.0 / m : 0.0) - cxx / inert;
    }
  const double* Ri = frame + 9 * (size_t)ci;
  const double* Rj = frame + 9 * (size_t)cj;
  double KR[3][3];
  for (int r = 0; r < 3; r++)
    for (int q = 0; q < 3; q++) KR[r][q] = K[r][0] * Rj[3 * q + 0] + K[r][1] * Rj[3 * q + 1] + K[r][2] * Rj[3 * q + 2];
  const double sg = si * sj;
  for (int r = 0; r < 3; r++)
    for (int q = 0; q < 3; q++) {
      const double v = Ri[3 * r + 0] * KR[0][q] + Ri[3 * r + 1] * KR[1][q] + Ri[3 * r + 2] * KR[2][q];
      W[r + 3 * q] += sg * v;
    }
}

__global__ void k_row_fill(int nc, const int* __restrict__ A, const int* __restrict__ B,
                           const long long* __restrict__ bptr, const int* __restrict__ blist,
                           const long long* __restrict__ rowptr, long long* __restrict__ colidx,
                           double* __restrict__ blocks, const double* __restrict__ frame,
                           const double* __restrict__ cpt, const double* __restrict__ bpos,
                           const double* __restrict__ mass, const double* __restrict__ inert) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    long long k = rowptr[c];
    const int bodies[2] = {A[c], B[c]};
    row_columns(c, A, B, bptr, blist, [&](int j) {
      double W[9];
      for (int e = 0; e < 9; e++) W[e] = 0.0;
      for (int t = 0; t < 2; t++) {
        const int b = bodies[t];
        if (b < 0) continue;
        if (A[j] == b || B[j] == b) add_body_block(c, j, b, B, frame, cpt, bpos, mass[b], inert[b], W);
      }
      for (int e = 0; e < 9; e++) blocks[9 * k + e] = W[e];
      colidx[k] = j;
      k++;
    });
  }
}

// q = H (v + h g), g = -9.81 e_z, in the generator's operation order.
__global__ void k_assemble_q(int nc, const int* __restrict__ A, const int* __restrict__ B,
                             const double* __restrict__ frame, const double* __restrict__ cpt,
                             const double* __restrict__ bpos, const double* __restrict__ vel, double h,
                             double* __restrict__ q) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    double u[3] = {0.0, 0.0, 0.0};
    const int bodies[2] = {A[c], B[c]};
    for (int t = 0; t < 2; t++) {
      const int b = bodies[t];
      if (b < 0) continue;
      const double s = (B[c] == b) ? 1.0 : -1.0;
      double d[3];
      for (int a = 0; a < 3; a++) d[a] = cpt[3 * (size_t)c + a] - bpos[3 * (size_t)b + a];
      const double* v = vel + 6 * (size_t)b;
      const double vf[3] = {v[0], v[1], v[2] - 9.81 * h};
      const double w[3] = {v[3], v[4], v[5]};
      const double wxd[3] = {w[1] * d[2] - w[2] * d[1], w[2] * d[0] - w[0] * d[2], w[0] * d[1] - w[1] * d[0]};
      for (int a = 0; a < 3; a++) u[a] += s * (vf[a] + wxd[a]);
    }
    const double* R = frame + 9 * (size_t)c;
    for (int r = 0; r < 3; r++) q[3 * (size_t)c + r] = R[3 * r + 0] * u[0] + R[3 * r + 1] * u[1] + R[3 * r + 2] * u[2];
  }
}

// v += std N(0, 1) per degree of freedom; normals by the Box-Muller method
// from two uniforms hashed (splitmix64) from (seed, index).
__device__ __forceinline__ unsigned long long splitmix(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

__global__ void k_random_walk(long long n, unsigned long long seed, double std, double* __restrict__ vel) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long x = splitmix(seed ^ splitmix((unsigned long long)i));
    const unsigned long long y = splitmix(x);
    const double u1 = ((double)(x >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    const double u2 = (double)(y >> 11) * (1.0 / 9007199254740992.0);
    vel[i] += std * (sqrt(-2.0 * log(u1)) * cospi(2.0 * u2));
  }
}

// sum of squares in fixed order: per-block partials, then one block
__global__ void k_sumsq_partial(long long n, const double* __restrict__ x, double* __restrict__ part) {
  __shared__ double sh[256];
  double t = 0.0;
  for (long long i = blockIdx.x * 256LL + threadIdx.x; i < n; i += 256LL * gridDim.x) t += x[i] * x[i];
  sh[threadIdx.x] = t;
  __syncthreads();
  for (int o = 128; o >= 1; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_sumsq_final(int nparts, double* __restrict__ part) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < nparts; k++) t += part[k];
    part[nparts] = t;
  }
}

}  // namespace fc3dgpu

static int assemble_q(fc3dgpu_ctx* c) {
  using namespace fc3dgpu;
  cudaStream_t s = c->stream;
  const int nc = c->nc;
  CK(ensure(&c->qo, &c->qo_cap, (size_t)nc * 3));
  k_assemble_q<<<grid1d(nc), 256, 0, s>>>(nc, c->cbA, c->cbB, c->cframe, c->cpoint, c->bpos, c->bvel, c->step_h,
                                          c->qo);
  k_set_q_mu<<<grid1d(nc), 256, 0, s>>>(nc, c->iperm, c->qo, c->muo, c->q64, c->mu64, c->q32, c->mu32);
  const int parts = 1024;
  CK(ensure(&c->qsum, &c->qsum_cap, (size_t)parts + 1));
  k_sumsq_partial<<<parts, 256, 0, s>>>(3LL * nc, c->qo, c->qsum);
  k_sumsq_final<<<1, 32, 0, s>>>(parts, c->qsum);
  CK(cudaGetLastError());
  c->launches += 4;
  double s2 = 0.0;
  CK(cudaMemcpyAsync(&s2, c->qsum + parts, sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  c->norm_q = sqrt(s2);
  c->have_q = true;
  return 0;
}

extern "C" int fc3dgpu_ctx_set_contacts(fc3dgpu_ctx* c, int nbodies, int ncontacts, const int32_t* bodyA,
                                        const int32_t* bodyB, const double* frame, const double* point,
                                        const double* body_pos, const double* body_mass, const double* body_inertia,
                                        int colour_kind) {
  using namespace fc3dgpu;
  if (!c || nbodies <= 0 || ncontacts <= 0 || !bodyA || !bodyB || !frame || !point || !body_pos || !body_mass ||
      !body_inertia) {
    fc3dgpu_set_error("fc3dgpu_ctx_set_contacts: invalid argument");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (c->nscenes > 0 || c->batch_graph) {
    if (c->batch_graph) cudaGraphExecDestroy(c->batch_graph);
    c->batch_graph = nullptr;
    c->nscenes = 0;
  }
  for (int k = 0; k < ncontacts; k++) {
    if (bodyB[k] < 0 || bodyB[k] >= nbodies || bodyA[k] < -1 || bodyA[k] >= nbodies || bodyA[k] == bodyB[k]) {
      fc3dgpu_set_error("fc3dgpu_ctx_set_contacts: contact %d joins bodies %d and %d of %d", k, bodyA[k], bodyB[k],
                        nbodies);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
  }
  for (int b = 0; b < nbodies; b++)
    if (!(body_mass[b] > 0.0) || !(body_inertia[b] > 0.0)) {
      fc3dgpu_set_error("fc3dgpu_ctx_set_contacts: body %d needs a positive mass and inertia", b);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
  CK(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  const int nc = ncontacts, nb = nbodies;
  c->have_contacts = c->have_vel = false;
  CK(ensure(&c->cbA, &c->cbA_cap, (size_t)nc));
  CK(ensure(&c->cbB, &c->cbB_cap, (size_t)nc));
  CK(ensure(&c->cframe, &c->cframe_cap, (size_t)nc * 9));
  CK(ensure(&c->cpoint, &c->cpoint_cap, (size_t)nc * 3));
  CK(ensure(&c->bpos, &c->bpos_cap, (size_t)nb * 3));
  CK(ensure(&c->bmass, &c->bmass_cap, (size_t)nb));
  CK(ensure(&c->binert, &c->binert_cap, (size_t)nb));
  CK(ensure(&c->bvel, &c->bvel_cap, (size_t)nb * 6));
  CK(ensure(&c->bdeg, &c->bdeg_cap, (size_t)nb));
  CK(ensure(&c->bptr, &c->bptr_cap, (size_t)nb + 1));
  CK(ensure(&c->blist, &c->blist_cap, (size_t)nc * 2));
  CK(ensure(&c->crowlen, &c->crowlen_cap, (size_t)nc));
  CK(ensure(&c->scratch64, &c->scratch64_cap, 4));
  CK(cudaMemcpyAsync(c->cbA, bodyA, sizeof(int) * nc, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->cbB, bodyB, sizeof(int) * nc, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->cframe, frame, sizeof(double) * 9 * nc, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->cpoint, point, sizeof(double) * 3 * nc, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->bpos, body_pos, sizeof(double) * 3 * nb, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->bmass, body_mass, sizeof(double) * nb, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->binert, body_inertia, sizeof(double) * nb, cudaMemcpyHostToDevice, s));
  // body -> incident contacts (sorted), then the block rows
  CK(cudaMemsetAsync(c->bdeg, 0, sizeof(int) * nb, s));
  k_body_degree<<<grid1d(nc), 256, 0, s>>>(nc, c->cbA, c->cbB, c->bdeg);
  k_scan_excl<int><<<1, 1024, 0, s>>>(nb, c->bdeg, c->bptr, c->scratch64);
  CK(cudaMemcpyAsync(c->bptr + nb, c->scratch64, sizeof(long long), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemsetAsync(c->bdeg, 0, sizeof(int) * nb, s));
  k_body_fill<<<grid1d(nc), 256, 0, s>>>(nc, c->cbA, c->cbB, c->bptr, c->bdeg, c->blist);
  k_body_sort<<<grid1d(nb), 256, 0, s>>>(nb, c->bptr, c->blist);
  k_row_len<<<grid1d(nc), 256, 0, s>>>(nc, c->cbA, c->cbB, c->bptr, c->blist, c->crowlen);
  CK(ensure(&c->rowptr, &c->rowptr_cap, (size_t)nc + 1));
  k_scan_excl<int><<<1, 1024, 0, s>>>(nc, c->crowlen, c->rowptr, c->scratch64);
  CK(cudaMemcpyAsync(c->rowptr + nc, c->scratch64, sizeof(long long), cudaMemcpyDeviceToDevice, s));
  long long nnzb = 0;
  CK(cudaMemcpyAsync(&nnzb, c->scratch64, sizeof(long long), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  CK(cudaGetLastError());
  c->launches += 6;
  CK(ensure(&c->colidx, &c->colidx_cap, (size_t)nnzb));
  CK(ensure(&c->blocks, &c->blocks_cap, (size_t)nnzb * 9));
  k_row_fill<<<grid1d(nc), 256, 0, s>>>(nc, c->cbA, c->cbB, c->bptr, c->blist, c->rowptr, c->colidx, c->blocks,
                                        c->cframe, c->cpoint, c->bpos, c->bmass, c->binert);
  CK(cudaGetLastError());
  c->launches++;
  int rc = build_layout(c, nc, nnzb, colour_kind, 0, nullptr);
  if (rc) return rc;
  c->nb = nb;
  c->have_contacts = true;
  c->have_mu = false;
  return 0;
}

extern "C" int fc3dgpu_ctx_set_mu(fc3dgpu_ctx* c, const double* mu) {
  if (!c || !mu || !c->have_W) {
    fc3dgpu_set_error("fc3dgpu_ctx_set_mu: W not set or null input");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  CK(cudaSetDevice(c->device));
  CK(ensure(&c->muo, &c->muo_cap, (size_t)c->nc));
  CK(cudaMemcpyAsync(c->muo, mu, sizeof(double) * c->nc, cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->have_mu = true;
  if (c->have_contacts && c->have_vel) return assemble_q(c);
  return 0;
}

extern "C" int fc3dgpu_ctx_set_velocities(fc3dgpu_ctx* c, const double* vel, double h) {
  if (!c || !vel || !c->have_contacts || !c->have_mu) {
    fc3dgpu_set_error("fc3dgpu_ctx_set_velocities: contacts and mu must be set first");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpyAsync(c->bvel, vel, sizeof(double) * 6 * c->nb, cudaMemcpyHostToDevice, c->stream));
  c->step_h = h;
  c->have_vel = true;
  return assemble_q(c);
}

extern "C" int fc3dgpu_ctx_random_walk(fc3dgpu_ctx* c, uint64_t seed, double std) {
  using namespace fc3dgpu;
  if (!c || !c->have_vel) {
    fc3dgpu_set_error("fc3dgpu_ctx_random_walk: velocities not set");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  CK(cudaSetDevice(c->device));
  k_random_walk<<<grid1d(6LL * c->nb), 256, 0, c->stream>>>(6LL * c->nb, (unsigned long long)seed, std, c->bvel);
  CK(cudaGetLastError());
  c->launches++;
  return assemble_q(c);
}

extern "C" int fc3dgpu_ctx_get_q(fc3dgpu_ctx* c, double* q) {
  if (!c || !q || !c->have_q) return NUMERICS_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpyAsync(q, c->qo, sizeof(double) * 3 * c->nc, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

extern "C" int fc3dgpu_ctx_get_velocities(fc3dgpu_ctx* c, double* vel) {
  if (!c || !vel || !c->have_vel) return NUMERICS_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpyAsync(vel, c->bvel, sizeof(double) * 6 * c->nb, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

extern "C" int fc3dgpu_ctx_sizes(fc3dgpu_ctx* c, int* nc, long long* nnzb, int* ncolours) {
  if (!c) return NUMERICS_ERR_NULL_POINTER;
  if (nc) *nc = c->have_W ? c->nc : 0;
  if (nnzb) *nnzb = c->have_W ? c->nnzb : 0;
  if (ncolours) *ncolours = c->have_W ? c->ncol : 0;
  return 0;
}

extern "C" int fc3dgpu_ctx_get_W(fc3dgpu_ctx* c, int64_t* rowptr, int64_t* colidx, double* blocks) {
  if (!c || !c->have_W) return NUMERICS_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(c->device));
  if (rowptr)
    CK(cudaMemcpyAsync(rowptr, c->rowptr, sizeof(long long) * (c->nc + 1), cudaMemcpyDeviceToHost, c->stream));
  if (colidx)
    CK(cudaMemcpyAsync(colidx, c->colidx, sizeof(long long) * c->nnzb, cudaMemcpyDeviceToHost, c->stream));
  if (blocks)
    CK(cudaMemcpyAsync(blocks, c->blocks, sizeof(double) * 9 * c->nnzb, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

// ---------------------------------------------------------------------------
// New values of W on an unchanged block structure
// ---------------------------------------------------------------------------
namespace fc3dgpu {
__global__ void k_differs(long long n, const long long* __restrict__ a, const long long* __restrict__ b,
                          int* __restrict__ diff) {
  int d = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    d |= a[i] != b[i];
  if (__syncthreads_or(d) && threadIdx.x == 0) atomicOr(diff, 1);
}
}  // namespace fc3dgpu

static int update_W_impl(fc3dgpu_ctx* c, int nc, const int64_t* rowptr, const int64_t* colidx, BlockSource blocks,
                         int kind) {
  using namespace fc3dgpu;
  if (!c || nc <= 0 || !rowptr || !colidx || (!blocks.flat && !blocks.ptrs)) {
    fc3dgpu_set_error("fc3dgpu_ctx_update_W: invalid argument");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (!c->have_W || c->nscenes > 0 || c->have_contacts || nc != c->nc || rowptr[nc] != c->nnzb ||
      kind != c->colour_kind) {
    if (c->batch_graph) {
      cudaGraphExecDestroy(c->batch_graph);
      c->batch_graph = nullptr;
    }
    return set_W_impl(c, nc, rowptr, colidx, blocks, kind, 0, nullptr);
  }
  CK(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  const long long nnzb = c->nnzb;
  // compare the structure with the current one on the device; no kernel
  // indexes with the new arrays before they are found equal to the
  // validated ones
  CK(ensure(&c->wtmp, &c->wtmp_cap, (size_t)(nc + 1) + (size_t)nnzb));
  CK(ensure(&c->wdiff, &c->wdiff_cap, 1));
  CK(cudaMemcpyAsync(c->wtmp, rowptr, sizeof(long long) * (nc + 1), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->wtmp + nc + 1, colidx, sizeof(long long) * nnzb, cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(c->wdiff, 0, sizeof(int), s));
  k_differs<<<grid1d(nc + 1), 256, 0, s>>>(nc + 1, c->wtmp, c->rowptr, c->wdiff);
  k_differs<<<grid1d(nnzb), 256, 0, s>>>(nnzb, c->wtmp + nc + 1, c->colidx, c->wdiff);
  if (!c->diff_h) CK(cudaHostAlloc((void**)&c->diff_h, sizeof(int), cudaHostAllocDefault));
  *c->diff_h = 1;
  CK(cudaMemcpyAsync(c->diff_h, c->wdiff, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaGetLastError());
  c->launches += 2;
  // the new values go to c->blocks while the comparison runs (the host
  // checks and gathers the blocks meanwhile; the copies queue behind it)
  c->have_W = false;
  {
    int rc = upload_blocks(c, nnzb, blocks);
    if (rc) {
      cudaStreamSynchronize(s);
      return rc;
    }
  }
  CK(cudaStreamSynchronize(s));
  if (*c->diff_h) {
    // another structure: the full upload (the values again with it)
    if (c->batch_graph) {
      cudaGraphExecDestroy(c->batch_graph);
      c->batch_graph = nullptr;
    }
    return set_W_impl(c, nc, rowptr, colidx, blocks, kind, 0, nullptr);
  }
  // same structure: the new values into the existing layout
  const long long nw = c->nslots * 9 * FC3D_SLAB;
  k_fill_blocks<<<grid1d(c->npad, 128), 128, 0, s>>>(c->npad, c->perm, c->rowptr, c->colidx, c->blocks, c->iperm,
                                                     c->slab_off, c->W64, c->col, c->D64, c->rho64);
  k_to_f32<<<grid1d(nw), 256, 0, s>>>(nw, c->W64, c->W32);
  k_to_f32<<<grid1d((long long)c->nslab * 9 * 32), 256, 0, s>>>((long long)c->nslab * 9 * 32, c->D64, c->D32);
  k_to_f32<<<grid1d((long long)c->nslab * 2 * 32), 256, 0, s>>>((long long)c->nslab * 2 * 32, c->rho64, c->rho32);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  c->launches += 4;
  c->have_W = true;
  return 0;
}

extern "C" int fc3dgpu_ctx_update_W(fc3dgpu_ctx* c, int nc, const int64_t* rowptr, const int64_t* colidx,
                                    const double* blocks, int kind) {
  return update_W_impl(c, nc, rowptr, colidx, BlockSource{blocks, nullptr}, kind);
}

extern "C" int fc3dgpu_ctx_update_W_ptrs(fc3dgpu_ctx* c, int nc, const int64_t* rowptr, const int64_t* colidx,
                                         const double* const* block, int kind) {
  return update_W_impl(c, nc, rowptr, colidx, BlockSource{nullptr, block}, kind);
}
