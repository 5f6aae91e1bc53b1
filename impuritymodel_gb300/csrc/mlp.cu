// BF16 multilayer perceptron over occupation bitstrings on the 5th-generation tensor cores.
//
// The network ranks candidate product states during basis pruning (no counterpart in
// upstream impurityModel, whose expand_basis keeps every state of the closure,
// impurityModel/ed/finite.py:1696-1803).  Its GEMMs run on tcgen05 fed by the tensor memory
// accelerator: a producer thread keeps a ring of K tiles in flight (2-D bulk-tensor copies
// into shared memory, completion on one mbarrier per stage), and a second thread issues
// tcgen05.mma (kind::f16, BF16 operands, FP32 accumulator in tensor memory) on each tile as
// it lands, never waiting for the MMAs themselves; every tile's MMAs commit to the stage's
// second mbarrier, which hands the stage back to the producer for the tile S ahead.
// The accumulator is read back with tcgen05.ld for a fused epilogue (bias, ReLU, ReLU mask,
// transposed copies for the backward pass) with 16-byte stores.
//
// One primitive covers forward and backward: C[M][N] = A[M][K] * B[N][K]^T with A and B
// row-major ("K-major") BF16, K a multiple of 64, M a multiple of 128, N a multiple of 16.
// The tile width (256, 64 or 16 columns) is the widest that still gives most SMs a tile.
// Every mbarrier wait has an iteration limit after which the kernel records
// EDGPU_ERR_NOCONV, waits (bounded) for its copies and MMAs still in flight, frees its tensor
// memory and returns.
#include <cuda_bf16.h>

#include "common.cuh"
#include "tma.cuh"

namespace edgpu {

constexpr int kGemmThreads = 128;  // 4 warps: tensor-memory lanes 0-127 = tile rows
constexpr int kBM = 128, kBK = 64;
constexpr uint32_t kSwizzleAtom = 1024;  // 8 rows x 128 bytes: one repeat of the 128-byte swizzle
constexpr long long kWaitLimit = 1LL << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of a K-major operand in the 128-byte swizzled layout: rows
// of 64 BF16 (128 bytes) one after another, the 16-byte chunks of row r permuted by XOR with
// r % 8, groups of 8 rows 1024 bytes apart (SBO); the leading-dimension offset is unused in
// this layout (encoded as 1).  `saddr` is the tile base (1024-byte aligned) plus 32 bytes per
// 16-column K step.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;                     // LBO (unused)
  d |= (uint64_t)(kSwizzleAtom >> 4) << 32;   // SBO
  d |= (uint64_t)1 << 46;                     // descriptor version of the tcgen05 family
  d |= (uint64_t)2 << 61;                     // 128-byte swizzle; base offset 0
  return d;
}

// Instruction descriptor of kind::f16: D F32, A and B BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* m, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* m, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes) : "memory");
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

// Box {64 columns, box rows} of the 2-D BF16 tensor `map` at (column x, row y) into dst,
// 128-byte swizzled.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
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

// The barrier's next phase completes once every tcgen05 operation this thread issued so far
// has completed.
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
  int vec;                   // C, Y and mask 16-byte aligned: 16-byte row stores and loads
};

// Shared-memory ring of a 128 x BN tile.  One stage holds the K tile (64 columns) of A and of
// B, each one 2-D bulk-tensor box {64, rows} in the 128-byte swizzled layout (one 128-byte
// request per row), each 1024-byte aligned.  The narrow 16-column tiles run only where the
// grid is small (a few row tiles, long K: the weight gradients), so they keep 8 stages in
// flight; the wider ones 4 or 3 (two or one CTAs per SM).
template <int BN>
struct GemmTile {
  static constexpr int kStages = BN <= 16 ? 8 : (BN >= 256 ? 3 : 4);
  static constexpr uint32_t kABytes = kBM * kBK * 2;          // 16 KiB
  static constexpr uint32_t kBBytes = BN * kBK * 2;
  static constexpr uint32_t kStageBytes = kABytes + kBBytes;  // a multiple of 1 KiB
  static constexpr uint32_t kCols = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
  static constexpr size_t kSmem = (size_t)kStages * kStageBytes + 1024;  // + alignment of the ring
};

template <int EPI, int BN>
__global__ void __launch_bounds__(kGemmThreads, 1)
    gemm_bf16_tc_kernel(const __grid_constant__ CUtensorMap amap, const __grid_constant__ CUtensorMap bmap,
                        GemmArgs g) {
  using T = GemmTile<BN>;
  constexpr int S = T::kStages;
  extern __shared__ unsigned char sm[];
  __shared__ uint64_t full[S], empty[S], done;
  __shared__ uint32_t tmem_base;
  __shared__ int failed;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
  const uint32_t ring = (smem_u32(sm) + 1023u) & ~1023u;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(T::kCols)
                 : "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  const int ktiles = g.K / kBK;
  if (warp == 1) {
    if (lane == 0) {
      // producer: K tile t into stage t % S once the MMAs of tile t - S have released it
      int issued = 0;
      bool ok = true;
      for (int t = 0; t < ktiles; ++t) {
        const int s = t % S;
        if (t >= S && !mbar_wait(&empty[s], (uint32_t)(t / S - 1) & 1u)) {
          ok = false;
          break;
        }
        if (*reinterpret_cast<volatile int*>(&failed)) break;  // the MMA side gave up
        const uint32_t a = ring + (uint32_t)s * T::kStageBytes, b = a + T::kABytes;
        mbar_expect_tx(&full[s], T::kStageBytes);
        tma_load_2d(a, &amap, t * kBK, m0, &full[s]);
        tma_load_2d(b, &bmap, t * kBK, n0, &full[s]);
        ++issued;
      }
      if (!ok) atomicExch(&failed, 1);
      // every copy issued has landed before the CTA may exit (earlier tiles of a stage were
      // consumed before its last one was issued)
      for (int t = issued > S ? issued - S : 0; t < issued; ++t) mbar_wait(&full[t % S], (uint32_t)(t / S) & 1u);
    }
    __syncwarp();
  } else if (warp == 0) {
    if (lane == 0) {
      // MMA issuer: never waits for MMAs, so they queue back to back in the tensor pipe
      const uint32_t idesc = idesc_bf16(kBM, BN);
      bool ok = true;
      for (int kt = 0; kt < ktiles; ++kt) {
        const int s = kt % S;
        if (!mbar_wait(&full[s], (uint32_t)(kt / S) & 1u)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t a = ring + (uint32_t)s * T::kStageBytes, b = a + T::kABytes;
#pragma unroll
        for (int k16 = 0; k16 < kBK / 16; ++k16)
          mma_bf16(tmem, smem_desc_sw128(a + (uint32_t)k16 * 32u), smem_desc_sw128(b + (uint32_t)k16 * 32u), idesc,
                   (kt > 0 || k16 > 0) ? 1u : 0u);
        mma_commit(&empty[s]);  // releases the stage to the producer once these MMAs are done
      }
      mma_commit(&done);
      if (!ok) atomicExch(&failed, 1);
    }
    __syncwarp();
  }
  if (!mbar_wait(&done, 0u)) atomicExch(&failed, 1);
  __syncthreads();
  tc_fence_after();
  if (failed) {
    if (tid == 0) atomicExch(g.status, (int32_t)EDGPU_ERR_NOCONV);
  } else {
    // epilogue: warp w owns tensor-memory lanes (= tile rows) 32w .. 32w+31; M % 128 == 0
    // and N % BN == 0, so every row and column of the tile exists
    const int row = m0 + warp * 32 + lane;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c0 = 0; c0 < BN; c0 += 16) {
      float v[16];
      tmem_ld16(trow + (uint32_t)c0, v);
      const int col0 = n0 + c0;
      const int64_t off = (int64_t)row * g.N + col0;
      if (EPI == kEpiStoreF32) {
        if (g.vec) {
          float4* dst = reinterpret_cast<float4*>(g.C + off);
#pragma unroll
          for (int q = 0; q < 4; ++q) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        } else {
#pragma unroll
          for (int q = 0; q < 16; ++q) g.C[off + q] = v[q];
        }
        continue;
      }
      if (EPI == kEpiBiasRelu) {
#pragma unroll
        for (int q = 0; q < 16; ++q) v[q] = fmaxf(v[q] + g.bias[col0 + q], 0.0f);
      }
      if (EPI == kEpiReluMask) {
        uint32_t mw[8];
        if (g.vec) {
          const uint4* src = reinterpret_cast<const uint4*>(g.mask + off);
          const uint4 m_lo = src[0], m_hi = src[1];
          mw[0] = m_lo.x, mw[1] = m_lo.y, mw[2] = m_lo.z, mw[3] = m_lo.w;
          mw[4] = m_hi.x, mw[5] = m_hi.y, mw[6] = m_hi.z, mw[7] = m_hi.w;
        } else {
          const unsigned short* src = reinterpret_cast<const unsigned short*>(g.mask + off);
#pragma unroll
          for (int q = 0; q < 8; ++q) mw[q] = (uint32_t)src[2 * q] | ((uint32_t)src[2 * q + 1] << 16);
        }
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const float m = __uint_as_float(((mw[q >> 1] >> (16 * (q & 1))) & 0xFFFFu) << 16);  // BF16 -> FP32
          v[q] = m > 0.0f ? v[q] : 0.0f;
        }
      }
      uint32_t pk[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
        pk[q] = *reinterpret_cast<const uint32_t*>(&h);
      }
      if (g.vec) {
        uint4* dst = reinterpret_cast<uint4*>(g.Y + off);
        dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
      } else {
        unsigned short* dst = reinterpret_cast<unsigned short*>(g.Y + off);
#pragma unroll
        for (int q = 0; q < 16; ++q) dst[q] = (unsigned short)(pk[q >> 1] >> (16 * (q & 1)));
      }
      if (g.Yt) {
        unsigned short* dst = reinterpret_cast<unsigned short*>(g.Yt);
#pragma unroll
        for (int q = 0; q < 16; ++q)  // lanes write consecutive rows: 64-byte runs per warp
          dst[(int64_t)(col0 + q) * g.M + row] = (unsigned short)(pk[q >> 1] >> (16 * (q & 1)));
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(T::kCols) : "memory");
}

// [rows][K] row-major BF16 as a 2-D tensor map with box {64 columns, box_rows rows}, 128-byte
// swizzled in shared memory.
bool gemm_operand_map(CUtensorMap* map, const __nv_bfloat16* ptr, int K, int rows, int box_rows) {
  EncodeTiledFn enc = encode_tiled();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1u, 1u};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(ptr), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int EPI, int BN>
int launch_gemm(const GemmArgs& g, cudaStream_t s) {
  using T = GemmTile<BN>;
  alignas(64) CUtensorMap amap, bmap;
  if (!gemm_operand_map(&amap, g.A, g.K, g.M, kBM) || !gemm_operand_map(&bmap, g.B, g.K, g.N, BN))
    return EDGPU_ERR_CUDA;
  auto* kern = gemm_bf16_tc_kernel<EPI, BN>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::kSmem) != cudaSuccess)
    return EDGPU_ERR_CUDA;
  dim3 grid(g.M / kBM, g.N / BN);
  kern<<<grid, kGemmThreads, T::kSmem, s>>>(amap, bmap, g);
  note_launch();
  return check_launch();
}

// Widest tile (256, 64 or 16 columns dividing N) that still gives about four fifths of the SMs
// a tile; the narrowest that divides N otherwise.
int gemm_tile_width(int M, int N) {
  const int64_t want = (int64_t)grid_cap() * 4 / 5;
  for (int bn : {256, 64, 16})
    if (N % bn == 0 && (int64_t)(M / kBM) * (N / bn) >= want) return bn;
  return 16;
}

template <int EPI>
int launch_gemm_bn(const GemmArgs& g, cudaStream_t s) {
  switch (gemm_tile_width(g.M, g.N)) {
    case 256:
      return launch_gemm<EPI, 256>(g, s);
    case 64:
      return launch_gemm<EPI, 64>(g, s);
    default:
      return launch_gemm<EPI, 16>(g, s);
  }
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

int gemm_bf16(int epi, GemmArgs g, cudaStream_t s) {
  if (!g.A || !g.B || !g.status || g.M < 1 || g.N < 16 || g.K < kBK || g.K % kBK || g.N % 16 || g.M % kBM)
    return EDGPU_ERR_ARG;
  if (g.N / 16 > 65535) return EDGPU_ERR_ARG;  // grid.y = N / tile width
  if (!aligned16(g.A) || !aligned16(g.B)) return EDGPU_ERR_ARG;
  switch (epi) {
    case kEpiStoreF32:
      if (!g.C) return EDGPU_ERR_ARG;
      g.vec = aligned16(g.C);
      return launch_gemm_bn<kEpiStoreF32>(g, s);
    case kEpiBiasRelu:
      if (!g.Y || !g.bias) return EDGPU_ERR_ARG;
      g.vec = aligned16(g.Y);
      return launch_gemm_bn<kEpiBiasRelu>(g, s);
    case kEpiReluMask:
      if (!g.Y || !g.mask) return EDGPU_ERR_ARG;
      g.vec = aligned16(g.Y) && aligned16(g.mask);
      return launch_gemm_bn<kEpiReluMask>(g, s);
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

extern "C" int edgpu_gemm_tile_width(int M, int N) {
  if (M < kBM || M % kBM || N < 16 || N % 16 || N / 16 > 65535) return 0;
  return gemm_tile_width(M, N);
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
