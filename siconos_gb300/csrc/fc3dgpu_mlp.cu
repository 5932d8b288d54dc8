// Learned warm start: a per-contact MLP (17 -> 128 -> 128 -> 128 -> 3, ReLU)
// that proposes each contact's reaction from local features, trained on the
// GPU with BF16 tensor-core matrix products accumulating in FP32.
//
// Every product is a warp-level tile of mma.m16n8k16 (BF16 in, FP32
// accumulate): C[M x N] = A[M x K] * Bt[N x K]^T, both operands row-major
// with K contiguous in shared memory, so each fragment register is one
// 32-bit load.  A block of 4 warps takes a tile of 64 samples through all
// layers in shared memory:
//   forward   Z_l = A_{l-1} W_l + b_l, A_l = ReLU(Z_l)        (Bt = W_l^T)
//   backward  dA_{l-1} = dZ_l W_l^T                            (Bt = W_l)
//             dW_l^T = dZ_l^T A_{l-1} per tile, tiles summed in a fixed
//             order by the Adam kernel
// Adam keeps FP32 master weights; the BF16 copies (W^T for the forward, W for
// the backward) are refreshed by the same kernel.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "fc3dgpu_mlp.h"

extern "C" void fc3dgpu_set_error(const char* fmt, ...);

namespace fc3dgpu {
namespace mlp {

constexpr int TILE = 64;   // samples per block
constexpr int NT = 128;    // threads per block: 4 warps
constexpr int NIN = FC3DGPU_MLP_FEATURES, KIN = 32, H = 128, NOUT = FC3DGPU_MLP_OUTPUTS, KOUT = 16;
constexpr int LD = H + 8;      // row length (bf16) of 128-wide tiles, padded against bank conflicts
constexpr int LDI = KIN + 8;   // of the 32-wide input tile
constexpr int LDT = TILE + 8;  // of transposed tiles [unit][sample]

__host__ __device__ constexpr int layer_k(int l) { return l == 0 ? KIN : H; }
__host__ __device__ constexpr int layer_n(int l) { return l == 3 ? KOUT : H; }
__host__ __device__ constexpr int woff(int l) {
  return l == 0 ? 0 : l == 1 ? KIN * H + H : l == 2 ? (KIN * H + H) + (H * H + H) : (KIN * H + H) + 2 * (H * H + H);
}
__host__ __device__ constexpr int boff(int l) { return woff(l) + layer_k(l) * layer_n(l); }
constexpr int NPARAM = woff(3) + H * KOUT + KOUT;

__device__ __forceinline__ int layer_of(int p) {
  int l = 0;
  while (l < 3 && p >= woff(l + 1)) l++;
  return l;
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One warp: rows [m0, m0 + 16 MT) of C = A Bt^T over N columns (multiple of
// 8) and a reduction of K (multiple of 16).  acc[mt][nt][i] is element i of
// the m16n8 tile (mt, nt).
template <int MT, int N, int K>
__device__ __forceinline__ void warp_gemm(const __nv_bfloat16* A, int lda, const __nv_bfloat16* Bt, int ldb, int m0,
                                          float (&acc)[MT][N / 8][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int mt = 0; mt < MT; mt++)
#pragma unroll
    for (int nt = 0; nt < N / 8; nt++)
#pragma unroll
      for (int i = 0; i < 4; i++) acc[mt][nt][i] = 0.f;
#pragma unroll
  for (int k0 = 0; k0 < K; k0 += 16) {
    uint32_t a[MT][4];
#pragma unroll
    for (int mt = 0; mt < MT; mt++) {
      const __nv_bfloat16* ap = A + (size_t)(m0 + mt * 16 + g) * lda + k0 + 2 * t;
      a[mt][0] = ld32(ap);
      a[mt][1] = ld32(ap + 8 * lda);
      a[mt][2] = ld32(ap + 8);
      a[mt][3] = ld32(ap + 8 * lda + 8);
    }
#pragma unroll
    for (int nt = 0; nt < N / 8; nt++) {
      const __nv_bfloat16* bp = Bt + (size_t)(nt * 8 + g) * ldb + k0 + 2 * t;
      const uint32_t b0 = ld32(bp), b1 = ld32(bp + 8);
#pragma unroll
      for (int mt = 0; mt < MT; mt++) mma_bf16(acc[mt][nt], a[mt], b0, b1);
    }
  }
}

// accumulator element (mt, nt, i) -> row and column within the warp's tile
__device__ __forceinline__ int acc_row(int mt, int i) { return mt * 16 + ((threadIdx.x & 31) >> 2) + (i >= 2 ? 8 : 0); }
__device__ __forceinline__ int acc_col(int nt, int i) { return nt * 8 + 2 * (threadIdx.x & 3) + (i & 1); }

struct Smem {
  __nv_bfloat16 x[TILE * LDI];      // standardised input tile [sample][feature]
  __nv_bfloat16 act[3][TILE * LD];  // A_1..A_3 [sample][unit]
  __nv_bfloat16 wt[H * LD];         // W_l^T [N][K] of the current layer
  float bias[H];
};

struct SmemT {
  Smem f;
  __nv_bfloat16 dz[TILE * LD];  // dZ_l [sample][unit]
  __nv_bfloat16 dzt[H * LDT];   // dZ_l^T [unit][sample]
  __nv_bfloat16 at[H * LDT];    // A_{l-1}^T [unit][sample]
  __nv_bfloat16 w[H * LD];      // W_l [K][N]
  float out[TILE * NOUT];
  float red[NT];
};

__device__ __forceinline__ float std_feature(float v, const float* stats, int f) {
  return (v - stats[f]) / stats[NIN + f];
}
__device__ __forceinline__ float std_target(float v, const float* stats, int c) {
  return (v - stats[2 * NIN + c]) / stats[2 * NIN + NOUT + c];
}

// Forward pass of the block's tile (s.x filled); the 3 outputs of each
// sample (standardised units) go to out[sample][3].
__device__ void forward_tile(const __nv_bfloat16* __restrict__ wT, const float* __restrict__ params, Smem& s,
                             float* out) {
  const int w = threadIdx.x >> 5;
#pragma unroll 1
  for (int l = 0; l < 4; l++) {
    const int K = layer_k(l), N = layer_n(l);
    const __nv_bfloat16* src = wT + woff(l);
    for (int e = threadIdx.x; e < N * K; e += NT) s.wt[(e / K) * LD + (e % K)] = src[e];
    for (int e = threadIdx.x; e < N; e += NT) s.bias[e] = params[boff(l) + e];
    __syncthreads();
    if (l < 3) {
      float acc[1][H / 8][4];
      if (l == 0)
        warp_gemm<1, H, KIN>(s.x, LDI, s.wt, LD, w * 16, acc);
      else
        warp_gemm<1, H, H>(s.act[l - 1], LD, s.wt, LD, w * 16, acc);
#pragma unroll
      for (int nt = 0; nt < H / 8; nt++)
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const int r = w * 16 + acc_row(0, i), c = acc_col(nt, i);
          const float z = acc[0][nt][i] + s.bias[c];
          s.act[l][r * LD + c] = __float2bfloat16_rn(z > 0.f ? z : 0.f);
        }
    } else {
      float acc[1][KOUT / 8][4];
      warp_gemm<1, KOUT, H>(s.act[2], LD, s.wt, LD, w * 16, acc);
#pragma unroll
      for (int nt = 0; nt < KOUT / 8; nt++)
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const int r = w * 16 + acc_row(0, i), c = acc_col(nt, i);
          if (c < NOUT) out[r * NOUT + c] = acc[0][nt][i] + s.bias[c];
        }
    }
    __syncthreads();
  }
}

// Proposals for samples [0, n): raw features X[n][17] -> Y[n][3] in the
// targets' units.
__global__ void __launch_bounds__(NT) k_infer(int n, const float* __restrict__ X, const __nv_bfloat16* __restrict__ wT,
                                              const float* __restrict__ params, const float* __restrict__ stats,
                                              float* __restrict__ Y) {
  extern __shared__ __align__(16) unsigned char smraw[];
  Smem& s = *reinterpret_cast<Smem*>(smraw);
  float* out = reinterpret_cast<float*>(smraw + sizeof(Smem));
  for (int tile = blockIdx.x; tile * TILE < n; tile += gridDim.x) {
    const int base = tile * TILE;
    for (int e = threadIdx.x; e < TILE * KIN; e += NT) {
      const int r = e / KIN, f = e % KIN;
      float v = 0.f;
      if (base + r < n && f < NIN) v = std_feature(X[(size_t)(base + r) * NIN + f], stats, f);
      s.x[r * LDI + f] = __float2bfloat16_rn(v);
    }
    __syncthreads();
    forward_tile(wT, params, s, out);
    for (int e = threadIdx.x; e < TILE * NOUT; e += NT) {
      const int r = e / NOUT, c = e % NOUT;
      if (base + r < n) Y[(size_t)(base + r) * NOUT + c] = out[e] * stats[2 * NIN + NOUT + c] + stats[2 * NIN + c];
    }
    __syncthreads();
  }
}

// One training tile (samples idx[64 b .. 64 b + 64) of the minibatch):
// forward, gradient of L = sum over the minibatch of |y - t|^2 / (3 nbatch)
// in standardised units, backward.  The tile's parameter gradient goes to
// grad[b][NPARAM] and its sum of squared errors to loss[b].
__global__ void __launch_bounds__(NT) k_train_tile(const float* __restrict__ X, const float* __restrict__ T,
                                                   int nsamples, const int* __restrict__ idx, int nbatch,
                                                   const __nv_bfloat16* __restrict__ wT,
                                                   const __nv_bfloat16* __restrict__ wK,
                                                   const float* __restrict__ params, const float* __restrict__ stats,
                                                   float* __restrict__ grad, float* __restrict__ loss) {
  extern __shared__ __align__(16) unsigned char smraw[];
  SmemT& s = *reinterpret_cast<SmemT*>(smraw);
  const int w = threadIdx.x >> 5;
  const int base = blockIdx.x * TILE;
  float* g = grad + (size_t)blockIdx.x * NPARAM;
  // a sample index outside the training set counts as an absent sample
  auto sample = [&](int r) -> int {
    if (base + r >= nbatch) return -1;
    const int i = idx[base + r];
    return (i >= 0 && i < nsamples) ? i : -1;
  };
  for (int e = threadIdx.x; e < TILE * KIN; e += NT) {
    const int r = e / KIN, f = e % KIN;
    float v = 0.f;
    const int i = sample(r);
    if (i >= 0 && f < NIN) v = std_feature(X[(size_t)i * NIN + f], stats, f);
    s.f.x[r * LDI + f] = __float2bfloat16_rn(v);
  }
  __syncthreads();
  forward_tile(wT, params, s.f, s.out);
  float lsum = 0.f;
  for (int e = threadIdx.x; e < TILE * KOUT; e += NT) {
    const int r = e / KOUT, c = e % KOUT;
    float d = 0.f;
    const int i = c < NOUT ? sample(r) : -1;
    if (i >= 0) {
      const float diff = s.out[r * NOUT + c] - std_target(T[(size_t)i * NOUT + c], stats, c);
      lsum += diff * diff;
      d = 2.f * diff / (float)(NOUT * nbatch);
    }
    const __nv_bfloat16 db = __float2bfloat16_rn(d);
    s.dz[r * LD + c] = db;
    s.dzt[c * LDT + r] = db;
  }
  s.red[threadIdx.x] = lsum;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int k = 0; k < NT; k++) t += s.red[k];
    loss[blockIdx.x] = t;
  }
#pragma unroll 1
  for (int l = 3; l >= 0; l--) {
    const int K = layer_k(l), N = layer_n(l);
    // bias gradient: column sums of dZ over the tile's samples, in order
    for (int c = threadIdx.x; c < N; c += NT) {
      float t = 0.f;
      for (int r = 0; r < TILE; r++) t += __bfloat162float(s.dzt[c * LDT + r]);
      g[boff(l) + c] = t;
    }
    const __nv_bfloat16* Ap = l == 0 ? s.f.x : s.f.act[l - 1];
    const int lda = l == 0 ? LDI : LD;
    for (int e = threadIdx.x; e < TILE * K; e += NT) {
      const int r = e / K, k = e % K;
      s.at[k * LDT + r] = Ap[r * lda + k];
    }
    __syncthreads();
    // dW^T [N][K] = dZ^T [N][samples] (A^T [K][samples])^T
    if (l == 3) {
      if (w == 0) {
        float acc[1][H / 8][4];
        warp_gemm<1, H, TILE>(s.dzt, LDT, s.at, LDT, 0, acc);
#pragma unroll
        for (int nt = 0; nt < H / 8; nt++)
#pragma unroll
          for (int i = 0; i < 4; i++) {
            const int nrow = acc_row(0, i), kcol = acc_col(nt, i);
            g[woff(l) + kcol * KOUT + nrow] = acc[0][nt][i];
          }
      }
    } else if (l == 0) {
      float acc[2][KIN / 8][4];
      warp_gemm<2, KIN, TILE>(s.dzt, LDT, s.at, LDT, w * 32, acc);
#pragma unroll
      for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < KIN / 8; nt++)
#pragma unroll
          for (int i = 0; i < 4; i++) {
            const int nrow = w * 32 + acc_row(mt, i), kcol = acc_col(nt, i);
            g[woff(l) + kcol * H + nrow] = acc[mt][nt][i];
          }
    } else {
      float acc[2][H / 8][4];
      warp_gemm<2, H, TILE>(s.dzt, LDT, s.at, LDT, w * 32, acc);
#pragma unroll
      for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < H / 8; nt++)
#pragma unroll
          for (int i = 0; i < 4; i++) {
            const int nrow = w * 32 + acc_row(mt, i), kcol = acc_col(nt, i);
            g[woff(l) + kcol * H + nrow] = acc[mt][nt][i];
          }
    }
    if (l == 0) break;
    // dA_{l-1} [samples][K] = dZ [samples][N] (W [K][N])^T, masked by ReLU'
    const __nv_bfloat16* src = wK + woff(l);
    for (int e = threadIdx.x; e < K * N; e += NT) s.w[(e / N) * LD + (e % N)] = src[e];
    __syncthreads();
    float acc[1][H / 8][4];
    if (l == 3)
      warp_gemm<1, H, KOUT>(s.dz, LD, s.w, LD, w * 16, acc);
    else
      warp_gemm<1, H, H>(s.dz, LD, s.w, LD, w * 16, acc);
    __syncthreads();  // every warp has read dz and dzt of layer l
#pragma unroll
    for (int nt = 0; nt < H / 8; nt++)
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const int r = w * 16 + acc_row(0, i), c = acc_col(nt, i);
        const bool on = __bfloat162float(s.f.act[l - 1][r * LD + c]) > 0.f;
        const __nv_bfloat16 v = __float2bfloat16_rn(on ? acc[0][nt][i] : 0.f);
        s.dz[r * LD + c] = v;
        s.dzt[c * LDT + r] = v;
      }
    __syncthreads();
  }
}

// Sum of the tiles' gradients in tile order, Adam on the FP32 master
// parameters (decoupled weight decay on weights), BF16 copies refreshed.
// lr == 0 only sums (gsum).
__global__ void k_adam(int ntiles, const float* __restrict__ grad, float* __restrict__ params, float* __restrict__ m1,
                       float* __restrict__ m2, __nv_bfloat16* __restrict__ wT, __nv_bfloat16* __restrict__ wK,
                       float lr, float wd, float bc1, float bc2, float* __restrict__ gsum) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < NPARAM; p += gridDim.x * blockDim.x) {
    float gs = 0.f;
    for (int t = 0; t < ntiles; t++) gs += grad[(size_t)t * NPARAM + p];
    if (gsum) gsum[p] = gs;
    if (lr == 0.f) continue;
    const int l = layer_of(p);
    const bool is_w = p < boff(l);
    const float a = b1 * m1[p] + (1.f - b1) * gs;
    const float v = b2 * m2[p] + (1.f - b2) * gs * gs;
    m1[p] = a;
    m2[p] = v;
    float np_ = params[p] - lr * (a / bc1) / (sqrtf(v / bc2) + eps);
    if (is_w) np_ -= lr * wd * params[p];
    params[p] = np_;
    if (is_w) {
      const int K = layer_k(l), N = layer_n(l), e = p - woff(l), k = e / N, nn = e % N;
      wK[woff(l) + k * N + nn] = __float2bfloat16_rn(np_);
      wT[woff(l) + nn * K + k] = __float2bfloat16_rn(np_);
    }
  }
}

__global__ void k_refresh_bf16(const float* __restrict__ params, __nv_bfloat16* __restrict__ wT,
                               __nv_bfloat16* __restrict__ wK) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < NPARAM; p += gridDim.x * blockDim.x) {
    const int l = layer_of(p);
    if (p >= boff(l)) continue;
    const int K = layer_k(l), N = layer_n(l), e = p - woff(l), k = e / N, nn = e % N;
    wK[woff(l) + k * N + nn] = __float2bfloat16_rn(params[p]);
    wT[woff(l) + nn * K + k] = __float2bfloat16_rn(params[p]);
  }
}

// ---------------------------------------------------------------------------
// Blackwell tensor-core path (tcgen05): the same network and the same
// arithmetic (BF16 operands, FP32 accumulation, BF16 activations) with every
// product issued as tcgen05.mma by one thread, accumulators in tensor memory
// (TMEM) and read back with tcgen05.ld.  A block is one warpgroup (4 warps)
// and takes 128 samples: each product is C[128][N] = A[128][K] B[N][K]^T
// with M = 128 (one TMEM lane per sample, warp w reading lanes 32w..32w+31),
// N = 16, 32 or 128, K a multiple of 16.  Operands sit in shared memory in
// the no-swizzle K-major layout of 8-row x 16-byte core matrices: element
// (r, k) of a tile with K columns at (r / 8) * 16 K + (k / 8) * 128 +
// (r % 8) * 16 + (k % 8) * 2 bytes, so the descriptors take a leading
// (K-direction) byte offset of 128 and a stride (8-row) byte offset of 16 K.
// The mma.sync kernels above stay as the checked reference path.
// ---------------------------------------------------------------------------
constexpr int TILE_TC = 128;
constexpr int NT_TC = 128;

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// element offset of (r, k) in a core-matrix tile with K columns
__device__ __forceinline__ int cm(int r, int k, int K) { return (r >> 3) * (K * 8) + (k >> 3) * 64 + (r & 7) * 8 + (k & 7); }

// shared-memory matrix descriptor: start address, leading and stride byte
// offsets (16-byte units), descriptor version 1 (bits 46-47), no swizzle
__device__ __forceinline__ uint64_t sdesc(const void* base, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((su32(base) & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= 1ull << 46;
  return d;
}

// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A and
// B BF16 (bits 7-9 = 1, 10-12 = 1), both K-major, N / 8 in bits 17-22, M / 16
// in bits 24-28
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
               : "memory");
}

__device__ __forceinline__ bool bar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(su32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Load 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

struct SmemTC {
  __nv_bfloat16 x[TILE_TC * KIN];      // standardised inputs, core layout, K = 32
  __nv_bfloat16 act[3][TILE_TC * H];   // A_1..A_3, core layout, K = 128
  __nv_bfloat16 w[H * H];              // W_l^T (forward), A_{l-1}^T then W_l (backward)
  __nv_bfloat16 dz[TILE_TC * H];       // dZ_l [sample][unit], core layout
  __nv_bfloat16 dzt[H * TILE_TC];      // dZ_l^T [unit][sample], core layout
  float out[TILE_TC * NOUT];
  float bias[H];
  float red[NT_TC];
  uint64_t bar;
  uint32_t tmem;
  int failed;
};
constexpr size_t SMEM_TC = sizeof(SmemTC);
static_assert(SMEM_TC <= 227 * 1024, "tensor-core tile must fit one block's shared memory");
static_assert(offsetof(SmemTC, act) % 128 == 0 && offsetof(SmemTC, w) % 128 == 0 && offsetof(SmemTC, dz) % 128 == 0 &&
                  offsetof(SmemTC, dzt) % 128 == 0,
              "operand tiles on 128-byte boundaries");

// Polls of the MMA completion barrier before a block gives up (and reports
// the failure through *status instead of waiting for ever).
constexpr unsigned long long TC_SPIN = 1ull << 26;

// One thread issues C = A B^T (M = 128) into TMEM and commits to the block's
// barrier; every thread then waits for it (bounded) and orders its later
// tcgen05.ld after the wait.  Returns false when the wait gave up.
__device__ __forceinline__ bool tc_gemm(SmemTC& s, uint32_t& phase, const __nv_bfloat16* A, const __nv_bfloat16* B,
                                        int N, int K) {
  proxy_fence();  // this thread's shared-memory writes, seen by the tensor cores
  __syncthreads();
  if (threadIdx.x == 0) {
    tc_fence_after();
    const uint32_t idesc = idesc_bf16(TILE_TC, N);
    for (int k0 = 0; k0 < K; k0 += 16)
      tc_mma(s.tmem, sdesc(A + k0 * 8, 128, (uint32_t)K * 16), sdesc(B + k0 * 8, 128, (uint32_t)K * 16), idesc,
             k0 > 0 ? 1u : 0u);
    tc_commit(&s.bar);
  }
  unsigned long long n = 0;
  bool ok = true;
  while (!bar_try(&s.bar, phase)) {
    if (++n > TC_SPIN) {
      ok = false;
      break;
    }
  }
  phase ^= 1u;
  ok = __syncthreads_and(ok) != 0;  // one decision for the whole block
  tc_fence_after();
  return ok;
}

// TMEM of the block (128 columns, warp 0 allocates) and its barrier.
__device__ __forceinline__ void tc_setup(SmemTC& s) {
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&s.tmem)), "r"(128)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(&s.bar)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s.failed = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
}

__device__ __forceinline__ void tc_teardown(SmemTC& s, int* status) {
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(s.tmem), "r"(128) : "memory");
  if (threadIdx.x == 0 && s.failed && status) atomicOr(status, 1);
}

// TMEM address of this thread's lane (sample) at column c
__device__ __forceinline__ uint32_t tlane(const SmemTC& s, int c) {
  return s.tmem + ((uint32_t)((threadIdx.x >> 5) * 32) << 16) + (uint32_t)c;
}

// Copy a [R][K] row-major BF16 matrix from global memory into a core tile.
__device__ __forceinline__ void to_core(__nv_bfloat16* dst, const __nv_bfloat16* __restrict__ src, int R, int K) {
  for (int e = threadIdx.x * 8; e < R * K; e += NT_TC * 8) {
    const int r = e / K, k = e % K;
    *reinterpret_cast<uint4*>(dst + cm(r, k, K)) = *reinterpret_cast<const uint4*>(src + e);
  }
}

// Forward pass of the block's 128-sample tile (s.x filled) with tcgen05;
// the 3 outputs of each sample (standardised) go to s.out.
__device__ bool forward_tile_tc(const __nv_bfloat16* __restrict__ wT, const float* __restrict__ params, SmemTC& s,
                                uint32_t& phase) {
  const int row = threadIdx.x;  // the thread's sample = its TMEM lane
#pragma unroll 1
  for (int l = 0; l < 4; l++) {
    const int K = layer_k(l), N = layer_n(l);
    to_core(s.w, wT + woff(l), N, K);
    for (int e = threadIdx.x; e < N; e += NT_TC) s.bias[e] = params[boff(l) + e];
    if (!tc_gemm(s, phase, l == 0 ? s.x : s.act[l - 1], s.w, N, K)) return false;
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tmem_ld16(tlane(s, c0), v);
      if (l < 3) {
        __align__(16) __nv_bfloat16 h[16];
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const float z = v[j] + s.bias[c0 + j];
          h[j] = __float2bfloat16_rn(z > 0.f ? z : 0.f);
        }
        *reinterpret_cast<uint4*>(s.act[l] + cm(row, c0, H)) = *reinterpret_cast<const uint4*>(h);
        *reinterpret_cast<uint4*>(s.act[l] + cm(row, c0 + 8, H)) = *reinterpret_cast<const uint4*>(h + 8);
      } else {
#pragma unroll
        for (int j = 0; j < NOUT; j++) s.out[row * NOUT + j] = v[j] + s.bias[j];
      }
    }
    tc_fence_before();
    __syncthreads();
  }
  return true;
}

// standardised features of sample i (or zeros) into row r of the input tile
__device__ __forceinline__ void load_x_row(SmemTC& s, int r, const float* __restrict__ X, long long i,
                                           const float* __restrict__ stats) {
  __align__(16) __nv_bfloat16 h[KIN];
#pragma unroll
  for (int f = 0; f < KIN; f++) {
    const float v = (i >= 0 && f < NIN) ? std_feature(X[(size_t)i * NIN + f], stats, f) : 0.f;
    h[f] = __float2bfloat16_rn(v);
  }
#pragma unroll
  for (int k0 = 0; k0 < KIN; k0 += 8)
    *reinterpret_cast<uint4*>(s.x + cm(r, k0, KIN)) = *reinterpret_cast<const uint4*>(h + k0);
}

__global__ void __launch_bounds__(NT_TC, 1) k_infer_tc(int n, const float* __restrict__ X,
                                                        const __nv_bfloat16* __restrict__ wT,
                                                        const float* __restrict__ params,
                                                        const float* __restrict__ stats, float* __restrict__ Y,
                                                        int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smraw_tc[];
  SmemTC& s = *reinterpret_cast<SmemTC*>(smraw_tc);
  tc_setup(s);
  uint32_t phase = 0;
  for (int tile = blockIdx.x; tile * TILE_TC < n; tile += gridDim.x) {
    const int base = tile * TILE_TC, r = threadIdx.x;
    load_x_row(s, r, X, base + r < n ? (long long)(base + r) : -1, stats);
    if (!forward_tile_tc(wT, params, s, phase)) {
      if (threadIdx.x == 0) s.failed = 1;
      break;
    }
    if (base + r < n)
      for (int c = 0; c < NOUT; c++)
        Y[(size_t)(base + r) * NOUT + c] = s.out[r * NOUT + c] * stats[2 * NIN + NOUT + c] + stats[2 * NIN + c];
    __syncthreads();
  }
  tc_teardown(s, status);
}

// One 128-sample training tile with tcgen05: as k_train_tile (same loss,
// same gradient layout grad[b][NPARAM], same loss[b]).
__global__ void __launch_bounds__(NT_TC, 1) k_train_tile_tc(const float* __restrict__ X, const float* __restrict__ T,
                                                             int nsamples, const int* __restrict__ idx, int nbatch,
                                                             const __nv_bfloat16* __restrict__ wT,
                                                             const __nv_bfloat16* __restrict__ wK,
                                                             const float* __restrict__ params,
                                                             const float* __restrict__ stats,
                                                             float* __restrict__ grad, float* __restrict__ loss,
                                                             int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smraw_tc[];
  SmemTC& s = *reinterpret_cast<SmemTC*>(smraw_tc);
  tc_setup(s);
  uint32_t phase = 0;
  const int base = blockIdx.x * TILE_TC, row = threadIdx.x;
  float* g = grad + (size_t)blockIdx.x * NPARAM;
  int si = -1;
  if (base + row < nbatch) {
    const int i = idx[base + row];
    si = (i >= 0 && i < nsamples) ? i : -1;  // outside the training set: an absent sample
  }
  load_x_row(s, row, X, si, stats);
  bool ok = forward_tile_tc(wT, params, s, phase);
  if (ok) {
    // output error: dZ_3 [sample][16] (K = 16) and its transpose [16][sample]
    float lsum = 0.f;
    __align__(16) __nv_bfloat16 h[KOUT];
#pragma unroll
    for (int c = 0; c < KOUT; c++) {
      float d = 0.f;
      if (c < NOUT && si >= 0) {
        const float diff = s.out[row * NOUT + c] - std_target(T[(size_t)si * NOUT + c], stats, c);
        lsum += diff * diff;
        d = 2.f * diff / (float)(NOUT * nbatch);
      }
      h[c] = __float2bfloat16_rn(d);
      s.dzt[cm(c, row, TILE_TC)] = h[c];
    }
    *reinterpret_cast<uint4*>(s.dz + cm(row, 0, KOUT)) = *reinterpret_cast<const uint4*>(h);
    *reinterpret_cast<uint4*>(s.dz + cm(row, 8, KOUT)) = *reinterpret_cast<const uint4*>(h + 8);
    s.red[threadIdx.x] = lsum;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.f;
      for (int k = 0; k < NT_TC; k++) t += s.red[k];
      loss[blockIdx.x] = t;
    }
  }
#pragma unroll 1
  for (int l = 3; l >= 0 && ok; l--) {
    const int K = layer_k(l), N = layer_n(l);
    // bias gradient: column sums of dZ over the tile's samples, in order
    for (int c = threadIdx.x; c < N; c += NT_TC) {
      float t = 0.f;
      for (int r = 0; r < TILE_TC; r++) t += __bfloat162float(s.dzt[cm(c, r, TILE_TC)]);
      g[boff(l) + c] = t;
    }
    // A_{l-1}^T [K][sample] into s.w
    const __nv_bfloat16* Ap = l == 0 ? s.x : s.act[l - 1];
    for (int k = 0; k < K; k++) s.w[cm(k, row, TILE_TC)] = Ap[cm(row, k, K)];
    // weight gradient, W_l [K][N] row-major in g
    if (l == 3) {
      // D [k][n] = A^T [k][s] (dZ^T [n][s])^T, M = K = 128, N = 16
      if (!(ok = tc_gemm(s, phase, s.w, s.dzt, KOUT, TILE_TC))) break;
      float v[16];
      tmem_ld16(tlane(s, 0), v);
#pragma unroll
      for (int j = 0; j < KOUT; j++) g[woff(3) + row * KOUT + j] = v[j];
    } else {
      // D [n][k] = dZ^T [n][s] (A^T [k][s])^T, M = N = 128, N = K
      if (!(ok = tc_gemm(s, phase, s.dzt, s.w, K, TILE_TC))) break;
      for (int c0 = 0; c0 < K; c0 += 16) {
        float v[16];
        tmem_ld16(tlane(s, c0), v);
#pragma unroll
        for (int j = 0; j < 16; j++) g[woff(l) + (c0 + j) * H + row] = v[j];
      }
    }
    tc_fence_before();
    __syncthreads();
    if (l == 0) break;
    // dA_{l-1} [s][K] = dZ [s][N] (W_l [K][N])^T, masked by ReLU'
    to_core(s.w, wK + woff(l), K, N);
    if (!(ok = tc_gemm(s, phase, s.dz, s.w, K, N))) break;
    __align__(16) __nv_bfloat16 nd[H];
    for (int c0 = 0; c0 < K; c0 += 16) {
      float v[16];
      tmem_ld16(tlane(s, c0), v);
#pragma unroll
      for (int j = 0; j < 16; j++) {
        const bool on = __bfloat162float(s.act[l - 1][cm(row, c0 + j, H)]) > 0.f;
        nd[c0 + j] = __float2bfloat16_rn(on ? v[j] : 0.f);
      }
    }
    tc_fence_before();
    __syncthreads();  // the product has read dz; every thread has its row of dA
#pragma unroll
    for (int c0 = 0; c0 < H; c0 += 8) *reinterpret_cast<uint4*>(s.dz + cm(row, c0, H)) = *reinterpret_cast<const uint4*>(nd + c0);
    for (int c = 0; c < H; c++) s.dzt[cm(c, row, TILE_TC)] = nd[c];
    __syncthreads();
  }
  if (!ok && threadIdx.x == 0) s.failed = 1;
  tc_teardown(s, status);
}

constexpr size_t SMEM_INFER = sizeof(Smem) + TILE * NOUT * sizeof(float);
constexpr size_t SMEM_TRAIN = sizeof(SmemT);
static_assert(SMEM_TRAIN <= 227 * 1024, "training tile must fit one block's shared memory");

}  // namespace mlp
}  // namespace fc3dgpu

// ---------------------------------------------------------------------------
// C-ABI (include/fc3dgpu_mlp.h)
// ---------------------------------------------------------------------------
using namespace fc3dgpu::mlp;

struct fc3dgpu_mlp {
  int device = 0;
  int sms = 0;
  cudaStream_t stream = nullptr;
  float* params = nullptr;
  float* m1 = nullptr;
  float* m2 = nullptr;
  __nv_bfloat16* wT = nullptr;
  __nv_bfloat16* wK = nullptr;
  float* stats = nullptr;
  float* grad = nullptr;
  float* gsum = nullptr;
  float* loss = nullptr;
  int* idx = nullptr;
  int grad_tiles = 0;
  float* X = nullptr;
  float* T = nullptr;
  size_t nsamples = 0, cap = 0;
  int step = 0;
  bool have_params = false;
  int tc = 1;              // products on tcgen05 (1, default) or mma.sync (0, the checked reference)
  int residual = 0;        // the network predicts the change of the reaction
  int* status = nullptr;   // nonzero: a tensor-core product did not complete
};

#define MCK(x)                                                                            \
  do {                                                                                    \
    cudaError_t e_ = (x);                                                                 \
    if (e_ != cudaSuccess) {                                                              \
      fc3dgpu_set_error("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
      return NUMERICS_ERR_UNKNOWN;                                                        \
    }                                                                                     \
  } while (0)

extern "C" int fc3dgpu_mlp_nparams(void) { return NPARAM; }

extern "C" void fc3dgpu_mlp_destroy(fc3dgpu_mlp* m) {
  if (!m) return;
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  void* ptrs[] = {m->params, m->m1, m->m2, m->wT, m->wK, m->stats, m->grad, m->gsum, m->loss, m->idx, m->X, m->T,
                  m->status};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

extern "C" fc3dgpu_mlp* fc3dgpu_mlp_create(int device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    fc3dgpu_set_error("fc3dgpu_mlp_create: no CUDA device %d", device);
    return nullptr;
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    fc3dgpu_set_error("fc3dgpu_mlp_create: cudaSetDevice(%d) failed", device);
    return nullptr;
  }
  fc3dgpu_mlp* m = new fc3dgpu_mlp();
  m->device = device;
  cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, device);
  bool ok = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaMalloc(&m->params, sizeof(float) * NPARAM) == cudaSuccess &&
            cudaMalloc(&m->m1, sizeof(float) * NPARAM) == cudaSuccess &&
            cudaMalloc(&m->m2, sizeof(float) * NPARAM) == cudaSuccess &&
            cudaMalloc(&m->gsum, sizeof(float) * NPARAM) == cudaSuccess &&
            cudaMalloc(&m->wT, sizeof(__nv_bfloat16) * NPARAM) == cudaSuccess &&
            cudaMalloc(&m->wK, sizeof(__nv_bfloat16) * NPARAM) == cudaSuccess &&
            cudaMalloc(&m->stats, sizeof(float) * FC3DGPU_MLP_STATS) == cudaSuccess &&
            cudaFuncSetAttribute(k_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_INFER) ==
                cudaSuccess &&
            cudaFuncSetAttribute(k_train_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TRAIN) ==
                cudaSuccess &&
            cudaFuncSetAttribute(k_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TC) == cudaSuccess &&
            cudaFuncSetAttribute(k_train_tile_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TC) ==
                cudaSuccess &&
            cudaMalloc(&m->status, sizeof(int)) == cudaSuccess && cudaMemset(m->status, 0, sizeof(int)) == cudaSuccess;
  if (!ok) {
    fc3dgpu_set_error("fc3dgpu_mlp_create: allocation or set-up failed (%s)", cudaGetErrorString(cudaGetLastError()));
    fc3dgpu_mlp_destroy(m);
    return nullptr;
  }
  return m;
}

extern "C" int fc3dgpu_mlp_set_params(fc3dgpu_mlp* m, const float* params, const float* stats) {
  if (!m || !params || !stats) return NUMERICS_ERR_NULL_POINTER;
  for (int f = 0; f < NIN + NOUT; f++) {
    const float sd = stats[f < NIN ? NIN + f : 2 * NIN + NOUT + (f - NIN)];
    if (!(sd > 0.f) || !isfinite(sd)) {
      fc3dgpu_set_error("fc3dgpu_mlp_set_params: standard deviation %d must be positive and finite", f);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
  }
  MCK(cudaSetDevice(m->device));
  MCK(cudaMemcpyAsync(m->params, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemcpyAsync(m->stats, stats, sizeof(float) * FC3DGPU_MLP_STATS, cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemsetAsync(m->m1, 0, sizeof(float) * NPARAM, m->stream));
  MCK(cudaMemsetAsync(m->m2, 0, sizeof(float) * NPARAM, m->stream));
  k_refresh_bf16<<<(NPARAM + 255) / 256, 256, 0, m->stream>>>(m->params, m->wT, m->wK);
  MCK(cudaGetLastError());
  MCK(cudaStreamSynchronize(m->stream));
  m->step = 0;
  m->have_params = true;
  return 0;
}

extern "C" int fc3dgpu_mlp_get_params(fc3dgpu_mlp* m, float* params, float* stats) {
  if (!m) return NUMERICS_ERR_NULL_POINTER;
  MCK(cudaSetDevice(m->device));
  if (params) MCK(cudaMemcpyAsync(params, m->params, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, m->stream));
  if (stats)
    MCK(cudaMemcpyAsync(stats, m->stats, sizeof(float) * FC3DGPU_MLP_STATS, cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  return 0;
}

extern "C" int fc3dgpu_mlp_set_data(fc3dgpu_mlp* m, size_t n, const float* X, const float* T) {
  if (!m || !X || !T) return NUMERICS_ERR_NULL_POINTER;
  if (n == 0 || n > (size_t)INT32_MAX) {
    fc3dgpu_set_error("fc3dgpu_mlp_set_data: %zu samples (1 to 2^31-1 allowed)", n);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  MCK(cudaSetDevice(m->device));
  if (n > m->cap) {
    MCK(cudaStreamSynchronize(m->stream));
    if (m->X) cudaFree(m->X);
    if (m->T) cudaFree(m->T);
    m->X = m->T = nullptr;
    m->cap = m->nsamples = 0;
    MCK(cudaMalloc(&m->X, sizeof(float) * NIN * n));
    MCK(cudaMalloc(&m->T, sizeof(float) * NOUT * n));
    m->cap = n;
  }
  MCK(cudaMemcpyAsync(m->X, X, sizeof(float) * NIN * n, cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemcpyAsync(m->T, T, sizeof(float) * NOUT * n, cudaMemcpyHostToDevice, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  m->nsamples = n;
  return 0;
}

static int tile_of(const fc3dgpu_mlp* m) { return m->tc ? TILE_TC : TILE; }

static int ensure_tiles(fc3dgpu_mlp* m, int tiles, int nbatch) {
  if (tiles <= m->grad_tiles && nbatch <= TILE * m->grad_tiles) return 0;
  if (tiles < (nbatch + TILE - 1) / TILE) tiles = (nbatch + TILE - 1) / TILE;
  MCK(cudaStreamSynchronize(m->stream));
  if (m->grad) cudaFree(m->grad);
  if (m->loss) cudaFree(m->loss);
  if (m->idx) cudaFree(m->idx);
  m->grad = m->loss = nullptr;
  m->idx = nullptr;
  m->grad_tiles = 0;
  MCK(cudaMalloc(&m->grad, sizeof(float) * NPARAM * (size_t)tiles));
  MCK(cudaMalloc(&m->loss, sizeof(float) * tiles));
  MCK(cudaMalloc(&m->idx, sizeof(int) * TILE * (size_t)tiles));
  m->grad_tiles = tiles;
  return 0;
}

// the device status word of the tensor-core kernels, read (and cleared) at a
// synchronisation point
static int check_status(fc3dgpu_mlp* m) {
  int st = 0;
  MCK(cudaMemcpyAsync(&st, m->status, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  if (st) {
    cudaMemsetAsync(m->status, 0, sizeof(int), m->stream);
    fc3dgpu_set_error("a tensor-core product of the warm-start network did not complete");
    return NUMERICS_ERR_UNKNOWN;
  }
  return 0;
}

static int launch_step(fc3dgpu_mlp* m, int nbatch, const int* idx_dev, float lr, float wd, bool keep_gsum) {
  const int tiles = (nbatch + tile_of(m) - 1) / tile_of(m);
  if (m->tc)
    k_train_tile_tc<<<tiles, NT_TC, SMEM_TC, m->stream>>>(m->X, m->T, (int)m->nsamples, idx_dev, nbatch, m->wT, m->wK,
                                                          m->params, m->stats, m->grad, m->loss, m->status);
  else
    k_train_tile<<<tiles, NT, SMEM_TRAIN, m->stream>>>(m->X, m->T, (int)m->nsamples, idx_dev, nbatch, m->wT, m->wK,
                                                       m->params, m->stats, m->grad, m->loss);
  MCK(cudaGetLastError());
  float bc1 = 1.f, bc2 = 1.f;
  if (lr != 0.f) {
    m->step++;
    bc1 = 1.f - powf(0.9f, (float)m->step);
    bc2 = 1.f - powf(0.999f, (float)m->step);
  }
  k_adam<<<(NPARAM + 255) / 256, 256, 0, m->stream>>>(tiles, m->grad, m->params, m->m1, m->m2, m->wT, m->wK, lr, wd,
                                                      bc1, bc2, keep_gsum ? m->gsum : nullptr);
  MCK(cudaGetLastError());
  return 0;
}

extern "C" int fc3dgpu_mlp_train_step(fc3dgpu_mlp* m, int nbatch, const int* idx, float lr, float wd,
                                      float* grad_out, float* loss_out, int apply) {
  if (!m || !idx) return NUMERICS_ERR_NULL_POINTER;
  if (!m->X || !m->have_params || nbatch <= 0) {
    fc3dgpu_set_error("fc3dgpu_mlp_train_step: parameters, training data and a positive batch are required");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  for (int k = 0; k < nbatch; k++)
    if (idx[k] < 0 || (size_t)idx[k] >= m->nsamples) {
      fc3dgpu_set_error("fc3dgpu_mlp_train_step: sample index %d out of range", idx[k]);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
  MCK(cudaSetDevice(m->device));
  const int tiles = (nbatch + tile_of(m) - 1) / tile_of(m);
  if (int rc = ensure_tiles(m, tiles, nbatch)) return rc;
  MCK(cudaMemcpyAsync(m->idx, idx, sizeof(int) * nbatch, cudaMemcpyHostToDevice, m->stream));
  if (int rc = launch_step(m, nbatch, m->idx, apply ? lr : 0.f, wd, grad_out != nullptr)) return rc;
  if (grad_out) MCK(cudaMemcpyAsync(grad_out, m->gsum, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, m->stream));
  std::vector<float> l(loss_out ? tiles : 0);
  if (loss_out) MCK(cudaMemcpyAsync(l.data(), m->loss, sizeof(float) * tiles, cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  if (int rc = check_status(m)) return rc;
  if (loss_out) {
    float s = 0.f;
    for (int t = 0; t < tiles; t++) s += l[t];
    *loss_out = s / (float)(NOUT * nbatch);
  }
  return 0;
}

extern "C" int fc3dgpu_mlp_train_step_device(fc3dgpu_mlp* m, int nbatch, const int* idx_dev, float lr, float wd) {
  if (!m || !idx_dev) return NUMERICS_ERR_NULL_POINTER;
  if (!m->X || !m->have_params || nbatch <= 0) {
    fc3dgpu_set_error("fc3dgpu_mlp_train_step_device: parameters, training data and a positive batch are required");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  MCK(cudaSetDevice(m->device));
  if (int rc = ensure_tiles(m, (nbatch + tile_of(m) - 1) / tile_of(m), nbatch)) return rc;
  return launch_step(m, nbatch, idx_dev, lr, wd, false);
}

static int infer_on(fc3dgpu_mlp* m, size_t n, const float* X, float* Y, cudaStream_t s) {
  if (n == 0) return 0;
  int grid = (int)((n + tile_of(m) - 1) / tile_of(m));
  const int cap = (m->tc ? 1 : 8) * (m->sms > 0 ? m->sms : 1);
  if (grid > cap) grid = cap;
  if (m->tc)
    k_infer_tc<<<grid, NT_TC, SMEM_TC, s>>>((int)n, X, m->wT, m->params, m->stats, Y, m->status);
  else
    k_infer<<<grid, NT, SMEM_INFER, s>>>((int)n, X, m->wT, m->params, m->stats, Y);
  MCK(cudaGetLastError());
  return 0;
}

extern "C" int fc3dgpu_mlp_infer_stream(fc3dgpu_mlp* m, size_t n, const float* X, float* Y, void* stream) {
  if (!m || (n > 0 && (!X || !Y))) return NUMERICS_ERR_NULL_POINTER;
  if (!m->have_params) {
    fc3dgpu_set_error("fc3dgpu_mlp_infer: no parameters loaded");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (n > (size_t)INT32_MAX) return NUMERICS_ERR_INVALID_ARGUMENT;
  MCK(cudaSetDevice(m->device));
  return infer_on(m, n, X, Y, static_cast<cudaStream_t>(stream));
}

extern "C" int fc3dgpu_mlp_infer(fc3dgpu_mlp* m, size_t n, const float* X, float* Y, int on_device) {
  if (!m || (n > 0 && (!X || !Y))) return NUMERICS_ERR_NULL_POINTER;
  if (!m->have_params) {
    fc3dgpu_set_error("fc3dgpu_mlp_infer: no parameters loaded");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (n == 0) return 0;
  if (n > (size_t)INT32_MAX) return NUMERICS_ERR_INVALID_ARGUMENT;
  MCK(cudaSetDevice(m->device));
  if (on_device) {
    if (int rc = infer_on(m, n, X, Y, m->stream)) return rc;
    MCK(cudaStreamSynchronize(m->stream));
    return check_status(m);
  }
  float *tx = nullptr, *ty = nullptr;
  MCK(cudaMalloc(&tx, sizeof(float) * NIN * n));
  if (cudaMalloc(&ty, sizeof(float) * NOUT * n) != cudaSuccess) {
    cudaFree(tx);
    fc3dgpu_set_error("fc3dgpu_mlp_infer: allocation failed");
    return NUMERICS_ERR_UNKNOWN;
  }
  int rc = 0;
  cudaError_t e = cudaMemcpyAsync(tx, X, sizeof(float) * NIN * n, cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) rc = infer_on(m, n, tx, ty, m->stream);
  if (e == cudaSuccess && !rc) e = cudaMemcpyAsync(Y, ty, sizeof(float) * NOUT * n, cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess && !rc) e = cudaStreamSynchronize(m->stream);
  cudaStreamSynchronize(m->stream);
  cudaFree(tx);
  cudaFree(ty);
  if (rc) return rc;
  MCK(e);
  return check_status(m);
}

extern "C" int fc3dgpu_mlp_set_residual(fc3dgpu_mlp* m, int residual) {
  if (!m) return NUMERICS_ERR_NULL_POINTER;
  const int prev = m->residual;
  m->residual = residual ? 1 : 0;
  return prev;
}

extern "C" int fc3dgpu_mlp_residual(const fc3dgpu_mlp* m) { return m ? m->residual : 0; }

extern "C" int fc3dgpu_mlp_set_tensor_path(fc3dgpu_mlp* m, int tcgen05) {
  if (!m) return NUMERICS_ERR_NULL_POINTER;
  const int prev = m->tc;
  m->tc = tcgen05 ? 1 : 0;
  return prev;
}
