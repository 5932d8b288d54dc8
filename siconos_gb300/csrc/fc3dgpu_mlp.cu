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
  void* ptrs[] = {m->params, m->m1, m->m2, m->wT, m->wK, m->stats, m->grad, m->gsum, m->loss, m->idx, m->X, m->T};
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
                cudaSuccess;
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

static int ensure_tiles(fc3dgpu_mlp* m, int tiles) {
  if (tiles <= m->grad_tiles) return 0;
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

static int launch_step(fc3dgpu_mlp* m, int nbatch, const int* idx_dev, float lr, float wd, bool keep_gsum) {
  const int tiles = (nbatch + TILE - 1) / TILE;
  k_train_tile<<<tiles, NT, SMEM_TRAIN, m->stream>>>(m->X, m->T, (int)m->nsamples, idx_dev, nbatch, m->wT, m->wK, m->params, m->stats,
                                                     m->grad, m->loss);
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
  const int tiles = (nbatch + TILE - 1) / TILE;
  if (int rc = ensure_tiles(m, tiles)) return rc;
  MCK(cudaMemcpyAsync(m->idx, idx, sizeof(int) * nbatch, cudaMemcpyHostToDevice, m->stream));
  if (int rc = launch_step(m, nbatch, m->idx, apply ? lr : 0.f, wd, grad_out != nullptr)) return rc;
  if (grad_out) MCK(cudaMemcpyAsync(grad_out, m->gsum, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, m->stream));
  std::vector<float> l(loss_out ? tiles : 0);
  if (loss_out) MCK(cudaMemcpyAsync(l.data(), m->loss, sizeof(float) * tiles, cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
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
  if (int rc = ensure_tiles(m, (nbatch + TILE - 1) / TILE)) return rc;
  return launch_step(m, nbatch, idx_dev, lr, wd, false);
}

static int infer_on(fc3dgpu_mlp* m, size_t n, const float* X, float* Y, cudaStream_t s) {
  if (n == 0) return 0;
  int grid = (int)((n + TILE - 1) / TILE);
  const int cap = 8 * (m->sms > 0 ? m->sms : 1);
  if (grid > cap) grid = cap;
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
    return 0;
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
  return 0;
}
