// BF16 multilayer perceptron over occupation bitstrings on the 5th-generation tensor cores.
//
// The network ranks candidate product states during basis pruning (no counterpart in
// upstream impurityModel, whose expand_basis keeps every state of the closure,
// impurityModel/ed/finite.py:1696-1803).  Its GEMMs run on tcgen05: one thread issues
// tcgen05.mma (kind::f16, BF16 operands, FP32 accumulator in tensor memory) on operand tiles
// staged in shared memory; the accumulator is read back with tcgen05.ld for a fused
// epilogue (bias, ReLU, ReLU mask, transposed copies for the backward pass).
//
// One primitive covers forward and backward: C[M][N] = A[M][K] * B[N][K]^T with A and B
// row-major ("K-major") BF16, K a multiple of 64, M a multiple of 128, N a multiple of 16
// and at most 256.  Every wait on the MMA completion barrier has an iteration limit after
// which the kernel records EDGPU_ERR_NOCONV, waits (bounded) once more, frees its tensor
// memory and returns.
#include <cuda_bf16.h>

#include "common.cuh"

namespace edgpu {

constexpr int kGemmThreads = 128;  // 4 warps: tensor-memory lanes 0-127 = tile rows
constexpr int kBM = 128, kBK = 64;
constexpr uint32_t kLBO = 128;   // bytes between core matrices adjacent along K
constexpr uint32_t kSBO = 1024;  // bytes between core matrices adjacent along M/N (8 K-chunks)
constexpr long long kWaitLimit = 1LL << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, no swizzle, K-major canonical layout: core matrices of
// 8 rows x 16 bytes stored contiguously, LBO apart along K and SBO apart along M/N.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((kLBO >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((kSBO >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of the tcgen05 family
  return d;                // base offset 0, absolute LBO mode, no swizzle
}

// Instruction descriptor of kind::f16: D F32, A and B BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* m, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* m, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(m)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Bounded wait for the given phase of the barrier; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* m, uint32_t phase) {
  for (long long t = 0; t < kWaitLimit; ++t)
    if (mbar_test(m, phase)) return true;
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* m) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(m))
               : "memory");
}

// 16 consecutive FP32 columns of this thread's tensor-memory lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

// Copy a [rows x 64] BF16 tile (row-major source, leading dimension ld elements) into the
// canonical no-swizzle K-major layout; rows past `valid` are zero.
__device__ __forceinline__ void stage_tile(unsigned char* dst, const __nv_bfloat16* src, int64_t ld, int rows,
                                           int valid) {
  for (int c = threadIdx.x; c < rows * 8; c += blockDim.x) {
    const int row = c >> 3, kc = c & 7;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (row < valid) v = *reinterpret_cast<const uint4*>(src + (int64_t)row * ld + kc * 8);
    *reinterpret_cast<uint4*>(dst + (row >> 3) * kSBO + kc * kLBO + (row & 7) * 16) = v;
  }
}

enum GemmEpilogue : int {
  kEpiStoreF32 = 0,   // C (float) = acc
  kEpiBiasRelu = 1,   // Y = relu(acc + bias[col]) -> BF16 Y[row][col] and Yt[col][row]
  kEpiReluMask = 2,   // Y = acc * (mask[row][col] > 0) -> BF16 Y and Yt
};

struct GemmArgs {
  const __nv_bfloat16* A;  // [M][K]
  const __nv_bfloat16* B;  // [N][K]
  int M, N, K;
  float* C;                  // kEpiStoreF32: [M][N]
  const float* bias;         // kEpiBiasRelu: [N]
  const __nv_bfloat16* mask; // kEpiReluMask: [M][N]
  __nv_bfloat16* Y;          // [M][N]
  __nv_bfloat16* Yt;         // [N][M] (may be null)
  int32_t* status;
};

template <int EPI, int BN>
__global__ void __launch_bounds__(kGemmThreads, 1) gemm_bf16_tc_kernel(GemmArgs g) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* sA = sm;                   // kBM x kBK bf16 = 16 KiB
  unsigned char* sB = sm + kBM * kBK * 2;   // BN x kBK bf16
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int failed;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
  constexpr uint32_t kCols = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(&mbar, 1);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = idesc_bf16(kBM, BN);
  const int ktiles = g.K / kBK;
  const int valid_a = min(kBM, g.M - m0), valid_b = min(BN, g.N - n0);
  uint32_t phase = 0;
  for (int kt = 0; kt < ktiles; ++kt) {
    stage_tile(sA, g.A + (int64_t)m0 * g.K + kt * kBK, g.K, kBM, valid_a);
    stage_tile(sB, g.B + (int64_t)n0 * g.K + kt * kBK, g.K, BN, valid_b);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic smem writes -> async proxy
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
#pragma unroll
      for (int k16 = 0; k16 < kBK / 16; ++k16)
        mma_bf16(tmem, smem_desc(a0 + k16 * 2 * kLBO), smem_desc(b0 + k16 * 2 * kLBO), idesc,
                 (kt > 0 || k16 > 0) ? 1u : 0u);
      mma_commit(&mbar);
    }
    // every thread waits: the tiles are overwritten next iteration, and the epilogue reads
    // the accumulator after the last one
    if (!mbar_wait(&mbar, phase)) failed = 1;
    phase ^= 1u;
    __syncthreads();
    if (failed) break;
  }
  tc_fence_after();
  if (failed) {
    if (tid == 0) {
      atomicExch(g.status, (int32_t)EDGPU_ERR_NOCONV);
      mbar_wait(&mbar, phase ^ 1u);  // bounded second chance for the MMAs in flight
    }
  } else {
    // epilogue: warp w owns tensor-memory lanes (= tile rows) 32w .. 32w+31
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < BN; c0 += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (row >= g.M) continue;
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int col = n0 + c0 + q;
        if (col >= g.N) break;
        float y = v[q];
        if (EPI == kEpiStoreF32) {
          g.C[(int64_t)row * g.N + col] = y;
          continue;
        }
        if (EPI == kEpiBiasRelu) y = fmaxf(y + g.bias[col], 0.0f);
        if (EPI == kEpiReluMask) y = (__bfloat162float(g.mask[(int64_t)row * g.N + col]) > 0.0f) ? y : 0.0f;
        const __nv_bfloat16 yb = __float2bfloat16_rn(y);
        g.Y[(int64_t)row * g.N + col] = yb;
        if (g.Yt) g.Yt[(int64_t)col * g.M + row] = yb;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
}

template <int EPI, int BN>
int launch_gemm(const GemmArgs& g, cudaStream_t s) {
  const size_t smem = (size_t)(kBM + BN) * kBK * 2 + 1024;
  // at least ~100 KiB per CTA keeps two CTAs per SM at most: 2 x 256 tensor-memory columns
  const size_t req = smem < 100 * 1024 ? 100 * 1024 : smem;
  auto* kern = gemm_bf16_tc_kernel<EPI, BN>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)req) != cudaSuccess)
    return EDGPU_ERR_CUDA;
  dim3 grid((g.M + kBM - 1) / kBM, (g.N + BN - 1) / BN);
  kern<<<grid, kGemmThreads, req, s>>>(g);
  note_launch();
  return check_launch();
}

int gemm_bf16(int epi, const GemmArgs& g, cudaStream_t s) {
  if (!g.A || !g.B || !g.status || g.M < 1 || g.N < 16 || g.K < kBK || g.K % kBK || g.N % 16 || g.M % kBM)
    return EDGPU_ERR_ARG;
  if (reinterpret_cast<uintptr_t>(g.A) % 16 || reinterpret_cast<uintptr_t>(g.B) % 16) return EDGPU_ERR_ARG;
  const int bn = g.N % 256 == 0 ? 256 : (g.N % 64 == 0 ? 64 : 16);
  switch (epi) {
    case kEpiStoreF32:
      if (!g.C) return EDGPU_ERR_ARG;
      return bn == 256 ? launch_gemm<kEpiStoreF32, 256>(g, s)
                       : (bn == 64 ? launch_gemm<kEpiStoreF32, 64>(g, s) : launch_gemm<kEpiStoreF32, 16>(g, s));
    case kEpiBiasRelu:
      if (!g.Y || !g.bias) return EDGPU_ERR_ARG;
      return bn == 256 ? launch_gemm<kEpiBiasRelu, 256>(g, s)
                       : (bn == 64 ? launch_gemm<kEpiBiasRelu, 64>(g, s) : launch_gemm<kEpiBiasRelu, 16>(g, s));
    case kEpiReluMask:
      if (!g.Y || !g.mask) return EDGPU_ERR_ARG;
      return bn == 256 ? launch_gemm<kEpiReluMask, 256>(g, s)
                       : (bn == 64 ? launch_gemm<kEpiReluMask, 64>(g, s) : launch_gemm<kEpiReluMask, 16>(g, s));
    default:
      return EDGPU_ERR_ARG;
  }
}

// ---------------------------------------------------------------------------------------
// Network pieces around the GEMMs (CUDA cores): input bits, output head, bias gradients,
// Adam, BF16 copies of the weights.
// ---------------------------------------------------------------------------------------

// X[b][i] = occupation of spin-orbital i (bit 63 - i%64 of word i/64) for i < n_in, BF16;
// Xt = X^T when not null.
__global__ void mlp_bits_kernel(const uint64_t* __restrict__ states, int W, int64_t B, int n_in,
                                __nv_bfloat16* __restrict__ X, __nv_bfloat16* __restrict__ Xt) {
  const int64_t total = B * (int64_t)n_in;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / n_in;
    const int i = (int)(t - b * n_in);
    const int q = i >> 6;
    float v = 0.0f;
    if (q < W) v = (float)((states[b * W + q] >> (63 - (i & 63))) & 1ull);
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    X[t] = h;
    if (Xt) Xt[(int64_t)i * B + b] = h;
  }
}

// y[b] = sum_j H[b][j] w3[j] + b3 (warp per row, FP32)
__global__ void mlp_head_kernel(const __nv_bfloat16* __restrict__ H, const float* __restrict__ w3, const float* b3,
                                int64_t B, int n_h, float* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  for (int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < B;
       b += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    float acc = 0.0f;
    for (int j = lane; j < n_h; j += 32) acc += __bfloat162float(H[b * n_h + j]) * w3[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[b] = acc + b3[0];
  }
}

// Mean-squared-error head backward: dy = 2 (y - t) / B; dH[b][j] = dy w3[j] (H[b][j] > 0)
// as BF16 dH and dHt; loss partials per block.
__global__ void mlp_head_backward_kernel(const __nv_bfloat16* __restrict__ H, const float* __restrict__ y,
                                         const float* __restrict__ target, const float* __restrict__ w3, int64_t B,
                                         int n_h, float* __restrict__ dy, __nv_bfloat16* __restrict__ dH,
                                         __nv_bfloat16* __restrict__ dHt) {
  const int64_t total = B * (int64_t)n_h;
  const float inv = 2.0f / (float)B;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / n_h;
    const int j = (int)(t - b * n_h);
    const float d = (y[b] - target[b]) * inv;
    if (j == 0) dy[b] = d;
    const float g = __bfloat162float(H[t]) > 0.0f ? d * w3[j] : 0.0f;
    const __nv_bfloat16 gb = __float2bfloat16_rn(g);
    dH[t] = gb;
    dHt[(int64_t)j * B + b] = gb;
  }
}

// out[r] = sum_c M[r][c] * (v ? v[c] : 1) for a row-major [rows][cols] BF16 matrix, block per
// row, fixed-order reduction (bias gradients from the transposed activations / deltas).
__global__ void mlp_row_dot_kernel(const __nv_bfloat16* __restrict__ M, int rows, int64_t cols,
                                   const float* __restrict__ v, float* __restrict__ out) {
  __shared__ float red[32];
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    float acc = 0.0f;
    for (int64_t c = threadIdx.x; c < cols; c += blockDim.x)
      acc += __bfloat162float(M[(int64_t)r * cols + c]) * (v ? v[c] : 1.0f);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.0f;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
      out[r] = t;
    }
    __syncthreads();
  }
}

// Adam on a flat FP32 parameter vector (bias-corrected step size lr_t from the host).
__global__ void mlp_adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                                float* __restrict__ v, int64_t n, float lr_t, float beta1, float beta2, float eps) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = beta1 * m[i] + (1.0f - beta1) * gi;
    const float vi = beta2 * v[i] + (1.0f - beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr_t * mi / (sqrtf(vi) + eps);
  }
}

// BF16 copy of a row-major [rows][cols] FP32 matrix, and of its transpose when Wt is set.
__global__ void mlp_to_bf16_kernel(const float* __restrict__ Wf, int rows, int cols, __nv_bfloat16* __restrict__ Wb,
                                   __nv_bfloat16* __restrict__ Wt) {
  const int64_t total = (int64_t)rows * cols;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t / cols), c = (int)(t - (int64_t)r * cols);
    const __nv_bfloat16 h = __float2bfloat16_rn(Wf[t]);
    if (Wb) Wb[t] = h;
    if (Wt) Wt[(int64_t)c * rows + r] = h;
  }
}

inline unsigned mlp_grid(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)grid_cap() * 8;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace edgpu

using namespace edgpu;

extern "C" int edgpu_gemm_bf16_epi(int epi, const void* A, const void* B, int M, int N, int K, float* C,
                                   const float* bias, const void* mask, void* Y, void* Yt, int32_t* status_dev,
                                   void* stream) {
  GemmArgs g{};
  g.A = reinterpret_cast<const __nv_bfloat16*>(A);
  g.B = reinterpret_cast<const __nv_bfloat16*>(B);
  g.M = M;
  g.N = N;
  g.K = K;
  g.C = C;
  g.bias = bias;
  g.mask = reinterpret_cast<const __nv_bfloat16*>(mask);
  g.Y = reinterpret_cast<__nv_bfloat16*>(Y);
  g.Yt = reinterpret_cast<__nv_bfloat16*>(Yt);
  g.status = status_dev;
  return gemm_bf16(epi, g, (cudaStream_t)stream);
}

extern "C" int edgpu_mlp_bits(const uint64_t* states, int W, int64_t B, int n_in, void* X, void* Xt, void* stream) {
  if (!states || W < 1 || B < 1 || n_in < 1 || !X) return EDGPU_ERR_ARG;
  mlp_bits_kernel<<<mlp_grid(B * n_in, 256), 256, 0, (cudaStream_t)stream>>>(
      states, W, B, n_in, reinterpret_cast<__nv_bfloat16*>(X), reinterpret_cast<__nv_bfloat16*>(Xt));
  note_launch();
  return check_launch();
}

extern "C" int edgpu_mlp_head(const void* H, const float* w3, const float* b3, int64_t B, int n_h, float* y,
                              void* stream) {
  if (!H || !w3 || !b3 || B < 1 || n_h < 1 || !y) return EDGPU_ERR_ARG;
  mlp_head_kernel<<<mlp_grid(B * 32, 256), 256, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const __nv_bfloat16*>(H), w3, b3, B, n_h, y);
  note_launch();
  return check_launch();
}

extern "C" int edgpu_mlp_head_backward(const void* H, const float* y, const float* target, const float* w3,
                                       int64_t B, int n_h, float* dy, void* dH, void* dHt, void* stream) {
  if (!H || !y || !target || !w3 || B < 1 || n_h < 1 || !dy || !dH || !dHt) return EDGPU_ERR_ARG;
  mlp_head_backward_kernel<<<mlp_grid(B * n_h, 256), 256, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const __nv_bfloat16*>(H), y, target, w3, B, n_h, dy, reinterpret_cast<__nv_bfloat16*>(dH),
      reinterpret_cast<__nv_bfloat16*>(dHt));
  note_launch();
  return check_launch();
}

extern "C" int edgpu_mlp_row_dot(const void* M, int rows, int64_t cols, const float* v, float* out, void* stream) {
  if (!M || rows < 1 || cols < 1 || !out) return EDGPU_ERR_ARG;
  mlp_row_dot_kernel<<<rows < 4096 ? rows : 4096, 256, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const __nv_bfloat16*>(M), rows, cols, v, out);
  note_launch();
  return check_launch();
}

extern "C" int edgpu_mlp_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr_t, float beta1,
                              float beta2, float eps, void* stream) {
  if (!p || !g || !m || !v || n < 1) return EDGPU_ERR_ARG;
  mlp_adam_kernel<<<mlp_grid(n, 256), 256, 0, (cudaStream_t)stream>>>(p, g, m, v, n, lr_t, beta1, beta2, eps);
  note_launch();
  return check_launch();
}

extern "C" int edgpu_mlp_to_bf16(const float* Wf, int rows, int cols, void* Wb, void* Wt, void* stream) {
  if (!Wf || rows < 1 || cols < 1 || (!Wb && !Wt)) return EDGPU_ERR_ARG;
  mlp_to_bf16_kernel<<<mlp_grid((int64_t)rows * cols, 256), 256, 0, (cudaStream_t)stream>>>(
      Wf, rows, cols, reinterpret_cast<__nv_bfloat16*>(Wb), reinterpret_cast<__nv_bfloat16*>(Wt));
  note_launch();
  return check_launch();
}

extern "C" int edgpu_gemm_bf16(const void* A, const void* B, int M, int N, int K, float* C, int32_t* status_dev,
                               void* stream) {
  GemmArgs g{};
  g.A = reinterpret_cast<const __nv_bfloat16*>(A);
  g.B = reinterpret_cast<const __nv_bfloat16*>(B);
  g.M = M;
  g.N = N;
  g.K = K;
  g.C = C;
  g.status = status_dev;
  return gemm_bf16(kEpiStoreF32, g, (cudaStream_t)stream);
}
