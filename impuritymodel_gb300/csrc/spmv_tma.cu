// Paged H·v with the x rows brought into shared memory by the tensor memory accelerator
// (edgpu_spmv_paged_tma_c64).
//
// Same pages as edgpu_spmv_paged (edgpu_spmv_pages_build): a page is a header column and
// slices of C = 32 / L row groups, one column holding one entry per group.  Here a column's C
// x rows are fetched by tile::gather4 bulk-tensor copies (four rows of a 2-D view of x per
// copy: [n rows][2R floats], box one row high) into a ring of `slots` column buffers per warp,
// each buffer with its mbarrier.  Lane 0 keeps `slots` columns in flight; the lanes wait on a
// column's barrier, read their 16 bytes of each group's row from shared memory and add the
// products.  The gathers thus cost one instruction per four rows and hold no registers, so
// many more x rows are in flight per SM than with per-lane loads.  Rows, columns and values
// come from the page in shared memory (cp.async), as in the per-lane form; each row sums its
// entries in the same order as there, so the two forms give the same y bit for bit.
//
// Waits are bounded: a barrier that does not complete within kWaitLimit polls sets the status
// word to EDGPU_ERR_NOCONV; the warp then waits (bounded again) for its own copies still in
// flight and stops.
#include "common.cuh"
#include "pages.cuh"
#include "tma.cuh"

namespace edgpu {
namespace {

constexpr int kTmaWarps = 4;
constexpr int kWaitLimit = 1 << 20;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// four rows r0..r3 of the 2-D tensor `map`, columns from 0, into dst (4 boxes, row after row)
__device__ __forceinline__ void tma_gather4(void* dst, const CUtensorMap* map, int r0, int r1, int r2, int r3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];\n" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(smem)), "l"(gmem) : "memory");
}

// Bytes of one warp's region: the ring (slots column buffers), the barriers, the page.
__host__ __device__ inline size_t tma_warp_bytes(int slots, int slot_bytes, int ch, int ent_bytes) {
  const size_t b = (size_t)slots * slot_bytes + (((size_t)8 * slots + 15) & ~(size_t)15) + (size_t)ch * ent_bytes;
  return (b + 127) & ~(size_t)127;
}

template <bool VALC, int R>
__global__ void __launch_bounds__(32 * kTmaWarps)
    spmv_pages_tma_kernel(int64_t n_pages, const Ent<float, VALC>* __restrict__ pages, int CH, int S,
                          const __grid_constant__ CUtensorMap xmap, float4* __restrict__ Y, int32_t* status) {
  using E = Ent<float, VALC>;
  constexpr int L = R / 2;             // lanes per entry: 16 bytes (two complex64 runs) each
  constexpr int C = 32 / L;            // row groups (entries per column)
  constexpr int G4 = (C + 3) / 4;      // gathers per column
  constexpr int ROWB = 8 * R;          // bytes of one x row
  constexpr int SLOTB = G4 * 4 * ROWB; // bytes of one column buffer
  extern __shared__ __align__(128) unsigned char tma_smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int grp = lane / L, sub = lane - grp * L;
  unsigned char* base = tma_smem + tma_warp_bytes(S, SLOTB, CH, (int)sizeof(E)) * wib;
  unsigned char* ring = base;
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + (size_t)S * SLOTB);
  E* pg = reinterpret_cast<E*>(base + (size_t)S * SLOTB + (((size_t)8 * S + 15) & ~(size_t)15));
  if (lane == 0) {
    for (int s = 0; s < S; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  }
  __syncwarp();
  unsigned phase = 0u;    // bit s: parity of the next completion of slot s
  unsigned pending = 0u;  // bit s: a gather of slot s is in flight (lane 0's view, kept by all)
  const int64_t nw = (int64_t)gridDim.x * kTmaWarps;
  const int chunks = CH * (int)sizeof(E) / 16;
  for (int64_t p = (int64_t)blockIdx.x * kTmaWarps + wib; p < n_pages; p += nw) {
    {
      const unsigned char* src = reinterpret_cast<const unsigned char*>(pages + p * CH);
      unsigned char* dst = reinterpret_cast<unsigned char*>(pg);
      for (int k = lane; k < chunks; k += 32) cp_async16(dst + 16 * k, src + 16 * k);
      asm volatile("cp.async.commit_group;\n" ::: "memory");
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
      __syncwarp();
    }
    const int ncols = pg[0].c;
    // lane 0: the gathers of column k into slot (k - 1) % S (header columns gather nothing)
    auto issue = [&](int k) {
      const int s = (k - 1) % S;
      if (pg[k * C].c <= -2) return;
      mbar_expect_tx(&bars[s], SLOTB);
#pragma unroll
      for (int g = 0; g < G4; ++g) {
        int r[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int e = 4 * g + q < C ? pg[k * C + 4 * g + q].c : -1;
          r[q] = e >= 0 ? e : 0;  // padding entries fetch row 0, never read
        }
        tma_gather4(ring + (size_t)s * SLOTB + (size_t)g * 4 * ROWB, &xmap, r[0], r[1], r[2], r[3], &bars[s]);
      }
    };
    const int first = ncols - 1 < S ? ncols - 1 : S;
    if (lane == 0)
      for (int k = 1; k <= first; ++k) issue(k);
    for (int k = 1; k <= first; ++k)
      if (pg[k * C].c > -2) pending |= 1u << ((k - 1) % S);
    __syncwarp();
    float ar[2] = {0.f, 0.f}, ai[2] = {0.f, 0.f};
    int64_t row = -1;
    bool heavy = false;
    auto flush = [&]() {  // called by the whole warp at the same column
      if (heavy) {
#pragma unroll
        for (int o = L; o < 32; o <<= 1)
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            ar[q] += __shfl_xor_sync(0xffffffffu, ar[q], o);
            ai[q] += __shfl_xor_sync(0xffffffffu, ai[q], o);
          }
      }
      if (row >= 0 && (!heavy || grp == 0)) __stcs(Y + row * L + sub, make_float4(ar[0], ai[0], ar[1], ai[1]));
      ar[0] = ar[1] = ai[0] = ai[1] = 0.f;
    };
    bool failed = false;
    for (int k = 1; k < ncols; ++k) {
      const int s = (k - 1) % S;
      const E e = pg[k * C + grp];
      if (e.c <= -2) {  // a slice header column (the same kind in every group)
        flush();
        row = e.c == INT_MIN ? -1 : (int64_t)(-2 - (int64_t)e.c);
        heavy = e.flag() != 0;
      } else {
        bool done = false;
        for (int it = 0; it < kWaitLimit && !done; ++it) done = __any_sync(0xffffffffu, mbar_try_wait(&bars[s], (phase >> s) & 1u));
        if (!done) {
          failed = true;
          break;
        }
        phase ^= 1u << s;
        pending &= ~(1u << s);
        if (e.c >= 0) {
          const float4 xv = *reinterpret_cast<const float4*>(ring + (size_t)s * SLOTB + (size_t)grp * ROWB + 16 * sub);
          float hr, hi = 0.f;
          if constexpr (VALC) {
            hr = e.vr;
            hi = e.vi;
          } else {
            hr = e.v;
          }
          ar[0] += hr * xv.x;
          ai[0] += hr * xv.y;
          ar[1] += hr * xv.z;
          ai[1] += hr * xv.w;
          if (VALC) {
            ar[0] -= hi * xv.y;
            ai[0] += hi * xv.x;
            ar[1] -= hi * xv.w;
            ai[1] += hi * xv.z;
          }
        }
      }
      __syncwarp();  // every lane has read slot s before it is refilled
      if (k + S < ncols) {
        if (lane == 0) issue(k + S);
        if (pg[(k + S) * C].c > -2) pending |= 1u << s;
      }
    }
    if (failed) {
      if (lane == 0) atomicExch(status, (int32_t)EDGPU_ERR_NOCONV);
      // the warp's own gathers still in flight, then stop (the product is incomplete)
      for (int s = 0; s < S; ++s) {
        if (!((pending >> s) & 1u)) continue;
        bool done = false;
        for (int it = 0; it < kWaitLimit && !done; ++it)
          done = __any_sync(0xffffffffu, mbar_try_wait(&bars[s], (phase >> s) & 1u));
      }
      return;
    }
    flush();
  }
}

template <bool VALC, int R>
int launch_tma(int64_t n_pages, const void* pages, int CH, int S, const CUtensorMap& map, float* y, int32_t* status,
               cudaStream_t s) {
  using E = Ent<float, VALC>;
  constexpr int C = 64 / R, G4 = (C + 3) / 4, SLOTB = G4 * 4 * 8 * R;
  const size_t smem = tma_warp_bytes(S, SLOTB, CH, (int)sizeof(E)) * kTmaWarps;
  if (smem > 200 * 1024) return EDGPU_ERR_ARG;
  if (cudaFuncSetAttribute(spmv_pages_tma_kernel<VALC, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return EDGPU_ERR_CUDA;
  int64_t blocks = (n_pages + kTmaWarps - 1) / kTmaWarps;
  const int64_t cap = (int64_t)grid_cap() * 16;
  if (blocks > cap) blocks = cap;
  spmv_pages_tma_kernel<VALC, R><<<(unsigned)blocks, 32 * kTmaWarps, smem, s>>>(
      n_pages, reinterpret_cast<const E*>(pages), CH, S, map, reinterpret_cast<float4*>(y), status);
  note_launch();
  return check_launch();
}

}  // namespace
}  // namespace edgpu

using namespace edgpu;

extern "C" int edgpu_spmv_paged_tma_c64(const edgpu_csr* h, const void* pages, int64_t n_pages, int page_entries,
                                        int slots, const float* x, float* y, int R, int32_t* status_dev,
                                        void* stream) {
  if (!h || !x || !y || !status_dev || h->n < 1 || n_pages < 0) return EDGPU_ERR_ARG;
  if (n_pages > 0 && !pages) return EDGPU_ERR_ARG;
  if (R != 4 && R != 8 && R != 16 && R != 32) return EDGPU_ERR_ARG;
  if (slots < 2 || slots > 32) return EDGPU_ERR_ARG;
  if (page_entries != 256 && page_entries != 512 && page_entries != 1024) return EDGPU_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y) | reinterpret_cast<uintptr_t>(pages)) & 15)
    return EDGPU_ERR_ARG;
  if (!h->val_cf && !h->val_rf) return EDGPU_ERR_ARG;
  if (h->n >= ((int64_t)1 << 31)) return EDGPU_ERR_ARG;  // gather row coordinates are 32-bit
  if (n_pages == 0) return EDGPU_OK;
  EncodeTiledFn enc = encode_tiled();
  if (!enc) return EDGPU_ERR_CUDA;
  // x as a 2-D tensor of floats: [n rows][2R], rows 8R bytes apart; box one row of 2R floats
  alignas(64) CUtensorMap map;
  const cuuint64_t dims[2] = {(cuuint64_t)(2 * R), (cuuint64_t)h->n};
  const cuuint64_t strides[1] = {(cuuint64_t)(8 * R)};
  const cuuint32_t box[2] = {(cuuint32_t)(2 * R), 1u};
  const cuuint32_t estr[2] = {1u, 1u};
  if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(x), dims, strides, box, estr,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return EDGPU_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  const bool cplx = h->val_cf != nullptr;
  switch (R) {
    case 4:
      return cplx ? launch_tma<true, 4>(n_pages, pages, page_entries, slots, map, y, status_dev, s)
                  : launch_tma<false, 4>(n_pages, pages, page_entries, slots, map, y, status_dev, s);
    case 8:
      return cplx ? launch_tma<true, 8>(n_pages, pages, page_entries, slots, map, y, status_dev, s)
                  : launch_tma<false, 8>(n_pages, pages, page_entries, slots, map, y, status_dev, s);
    case 16:
      return cplx ? launch_tma<true, 16>(n_pages, pages, page_entries, slots, map, y, status_dev, s)
                  : launch_tma<false, 16>(n_pages, pages, page_entries, slots, map, y, status_dev, s);
    default:
      return cplx ? launch_tma<true, 32>(n_pages, pages, page_entries, slots, map, y, status_dev, s)
                  : launch_tma<false, 32>(n_pages, pages, page_entries, slots, map, y, status_dev, s);
  }
}
