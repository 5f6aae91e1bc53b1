// Device radix sort of packed product states, prefix scans, segmented reduction, merge of
// sorted bases and batched binary search.  These replace the Python set/dict/sorted
// bookkeeping of upstream expand_basis (impurityModel/ed/finite.py:1696-1803) and the
// dict accumulation inside applyOp (finite.py:1355-1388).
#include "common.cuh"

namespace edgpu {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

// ---------------------------------------------------------------------------------------
// Exclusive scan of int64 (multi-level, reduce-then-scan)
// ---------------------------------------------------------------------------------------

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t* warp_tot, int64_t& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    int64_t t = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < nw) warp_tot[lane] = t;
  }
  __syncthreads();
  const int64_t before = warp ? warp_tot[warp - 1] : 0;
  total = warp_tot[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const int64_t* in, int64_t n, int64_t* partial) {
  __shared__ int64_t wt[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < n) s += in[base + k];
  int64_t total;
  block_exclusive_scan(s, wt, total);
  if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_down_kernel(const int64_t* in, int64_t n, const int64_t* block_off,
                                                                 int64_t* out) {
  __shared__ int64_t wt[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    s += v[k];
  }
  int64_t total;
  int64_t run = block_exclusive_scan(s, wt, total) + (block_off ? block_off[blockIdx.x] : 0);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) {
    out[n] = (block_off ? block_off[blockIdx.x] : 0) + total;
  }
}

static size_t scan_ws_elems(int64_t n) {
  if (n <= kScanTile) return 0;
  const int64_t nb = (n + kScanTile - 1) / kScanTile;
  return (size_t)(nb + 1) + scan_ws_elems(nb);
}

static int scan_rec(const int64_t* in, int64_t* out, int64_t n, int64_t* ws, cudaStream_t s) {
  const int64_t nb = (n + kScanTile - 1) / kScanTile;
  if (nb <= 1) {
    scan_down_kernel<<<1, kScanThreads, 0, s>>>(in, n, nullptr, out); note_launch();
    return check_launch();
  }
  int64_t* partial = ws;
  int64_t* partial_scan = ws + nb + 1;
  (void)partial_scan;
  scan_reduce_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, partial); note_launch();
  // Scan partial sums in place into a temp region after them: reuse a second level.
  int64_t* next_ws = ws + nb + 1;
  // The scan output of the partials needs nb + 1 entries; put it into `partial` itself via
  // a recursive call writing to the level's output buffer located in next level's space.
  int rc = scan_rec(partial, partial, nb, next_ws, s);
  if (rc) return rc;
  scan_down_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, partial, out); note_launch();
  return check_launch();
}

// ---------------------------------------------------------------------------------------
// Radix sort (stable LSD, 8-bit digits) of W-word keys with a uint32 payload
// ---------------------------------------------------------------------------------------

constexpr int kSortWarps = 16;
constexpr int kSortThreads = kSortWarps * 32;
constexpr int kSortRounds = 8;
constexpr int kSortTile = kSortThreads * kSortRounds;

template <int W>
__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(const uint64_t* keys, int64_t n, int q, int shift,
                                                                  int64_t* hist, int64_t nblocks) {
  __shared__ int h[256];
  for (int d = threadIdx.x; d < 256; d += blockDim.x) h[d] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kSortTile;
  for (int k = threadIdx.x; k < kSortTile; k += blockDim.x) {
    const int64_t i = base + k;
    if (i < n) {
      const int d = (int)((keys[i * W + q] >> shift) & 0xFF);
      atomicAdd(&h[d], 1);
    }
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(int64_t)d * nblocks + blockIdx.x] = h[d];
}

template <int W>
__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(const uint64_t* keys_in, const uint32_t* pay_in,
                                                                     uint64_t* keys_out, uint32_t* pay_out, int64_t n,
                                                                     int q, int shift, const int64_t* offs,
                                                                     int64_t nblocks) {
  __shared__ int cnt[kSortWarps][256];
  __shared__ int64_t gbase[256];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = threadIdx.x; k < kSortWarps * 256; k += blockDim.x) (&cnt[0][0])[k] = 0;
  __syncthreads();
  const int64_t wbase = (int64_t)blockIdx.x * kSortTile + (int64_t)warp * 32 * kSortRounds;
  const unsigned lt = (1u << lane) - 1u;
  for (int r = 0; r < kSortRounds; ++r) {
    const int64_t i = wbase + r * 32 + lane;
    const bool valid = i < n;
    const unsigned vmask = __ballot_sync(FULL, valid);
    if (valid) {
      const int d = (int)((keys_in[i * W + q] >> shift) & 0xFF);
      const unsigned peers = __match_any_sync(vmask, d);
      if (lane == __ffs(peers) - 1) cnt[warp][d] += __popc(peers);
    }
    __syncwarp();
  }
  __syncthreads();
  if (threadIdx.x < 256) {
    const int d = threadIdx.x;
    int run = 0;
    for (int w = 0; w < kSortWarps; ++w) {
      const int t = cnt[w][d];
      cnt[w][d] = run;
      run += t;
    }
    gbase[d] = offs[(int64_t)d * nblocks + blockIdx.x];
  }
  __syncthreads();
  for (int r = 0; r < kSortRounds; ++r) {
    const int64_t i = wbase + r * 32 + lane;
    const bool valid = i < n;
    const unsigned vmask = __ballot_sync(FULL, valid);
    int d = 0;
    unsigned peers = 0;
    int rank = 0;
    if (valid) {
      d = (int)((keys_in[i * W + q] >> shift) & 0xFF);
      peers = __match_any_sync(vmask, d);
      rank = cnt[warp][d] + __popc(peers & lt);
    }
    __syncwarp();
    if (valid) {
      const int64_t dst = gbase[d] + rank;
#pragma unroll
      for (int k = 0; k < W; ++k) keys_out[dst * W + k] = keys_in[i * W + k];
      pay_out[dst] = pay_in[i];
      if (lane == __ffs(peers) - 1) cnt[warp][d] += __popc(peers);
    }
    __syncwarp();
  }
}

template <int W>
__global__ void vary_kernel(const uint64_t* keys, int64_t n, unsigned long long* out) {
  uint64_t acc[W];
  uint64_t k0[W];
#pragma unroll
  for (int q = 0; q < W; ++q) {
    acc[q] = 0;
    k0[q] = keys[q];
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int q = 0; q < W; ++q) acc[q] |= keys[i * W + q] ^ k0[q];
  }
#pragma unroll
  for (int q = 0; q < W; ++q) {
    uint64_t v = acc[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v |= __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicOr(out + q, (unsigned long long)v);
  }
}

template <int W>
__global__ void copy_states_kernel(const uint64_t* src, const uint32_t* psrc, uint64_t* dst, uint32_t* pdst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int q = 0; q < W; ++q) dst[i * W + q] = src[i * W + q];
    pdst[i] = psrc[i];
  }
}

template <int W>
__global__ void heads_kernel(const uint64_t* keys, int64_t n, int64_t* head) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    head[i] = (i == 0) ? 1 : (state_cmp_mm<W>(keys + i * W, keys + (i - 1) * W) != 0 ? 1 : 0);
  }
}

template <int W>
__global__ void segment_reduce_kernel(const uint64_t* keys, const uint32_t* payload, int64_t n,
                                      const int64_t* head_scan, const double2* vals, uint64_t* out_keys,
                                      uint32_t* out_first, double2* out_vals) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = head_scan[i];
    if (head_scan[i + 1] == o) continue;  // not a head
#pragma unroll
    for (int q = 0; q < W; ++q) out_keys[o * W + q] = keys[i * W + q];
    if (out_first) out_first[o] = payload[i];
    if (vals && out_vals) {
      double2 acc = vals[payload[i]];
      for (int64_t j = i + 1; j < n && head_scan[j + 1] == head_scan[j]; ++j) {
        const double2 v = vals[payload[j]];
        acc.x = __dadd_rn(acc.x, v.x);
        acc.y = __dadd_rn(acc.y, v.y);
      }
      out_vals[o] = acc;
    }
  }
}

template <int W>
__global__ void merge_kernel(const uint64_t* a, int64_t na, const uint64_t* b, int64_t nb, uint64_t* out) {
  const int64_t tot = na + nb;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
    uint64_t key[W];
    int64_t pos;
    if (t < na) {
      load_state<W>(a + t * W, key);
      pos = t + lower_bound_state<W>(b, nb, key);
    } else {
      const int64_t k = t - na;
      load_state<W>(b + k * W, key);
      pos = k + lower_bound_state<W>(a, na, key);
    }
    store_state<W>(out + pos * W, key);
  }
}

template <int W>
__global__ void lookup_kernel(const uint64_t* basis, int64_t n, const uint64_t* query, int64_t nq, int64_t* out) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nq; t += (int64_t)gridDim.x * blockDim.x) {
    uint64_t key[W];
    load_state<W>(query + t * W, key);
    out[t] = find_state<W>(basis, n, key);
  }
}

inline unsigned grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)grid_cap() * 16;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace edgpu

using namespace edgpu;

extern "C" size_t edgpu_scan_workspace(int64_t n) { return scan_ws_elems(n) * sizeof(int64_t) + 256; }

extern "C" int edgpu_scan_i64(const int64_t* in, int64_t* out, int64_t n, void* workspace, size_t workspace_bytes,
                              void* stream) {
  if (n < 0 || !out) return EDGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (n == 0) {
    cudaMemsetAsync(out, 0, sizeof(int64_t), s);
    return check_launch();
  }
  if (!in) return EDGPU_ERR_ARG;
  if (workspace_bytes < edgpu_scan_workspace(n)) return EDGPU_ERR_WORKSPACE;
  return scan_rec(in, out, n, reinterpret_cast<int64_t*>(workspace), s);
}

namespace edgpu {

// ---------------------------------------------------------------------------------------
// Small inputs: one CTA sorts (key, original position) pairs in shared memory with a bitonic
// network (a total order, so the result is the stable sort), one launch instead of a
// histogram, scan and scatter launch per varying key byte.
// ---------------------------------------------------------------------------------------
constexpr int kSmallSortThreads = 1024;
constexpr size_t kSmallSortBytes = 160 * 1024;

inline int small_sort_pow2(int64_t n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

inline bool small_sort_fits(int n_words, int64_t n) {
  return n <= 8192 && (size_t)small_sort_pow2(n) * (8 * (size_t)n_words + 4) <= kSmallSortBytes;
}

template <int W>
__global__ void __launch_bounds__(kSmallSortThreads) small_sort_kernel(uint64_t* keys, uint32_t* payload, int n, int N) {
  extern __shared__ __align__(16) unsigned char sm[];
  uint64_t* k = reinterpret_cast<uint64_t*>(sm);
  uint32_t* idx = reinterpret_cast<uint32_t*>(k + (size_t)N * W);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
#pragma unroll
    for (int q = 0; q < W; ++q) k[(size_t)i * W + q] = i < n ? keys[(size_t)i * W + q] : ~0ull;
    idx[i] = (uint32_t)i;  // padding sorts last: all-ones keys, positions >= n
  }
  __syncthreads();
  for (int size = 2; size <= N; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = threadIdx.x; t < (N >> 1); t += blockDim.x) {
        const int lo = 2 * t - (t & (stride - 1));
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        int c = 0;
#pragma unroll
        for (int q = 0; q < W; ++q) {
          if (c == 0) {
            const uint64_t a = k[(size_t)lo * W + q], b = k[(size_t)hi * W + q];
            c = a < b ? -1 : (a > b ? 1 : 0);
          }
        }
        if (c == 0) c = idx[lo] < idx[hi] ? -1 : 1;
        if ((c > 0) == up) {
#pragma unroll
          for (int q = 0; q < W; ++q) {
            const uint64_t tmp = k[(size_t)lo * W + q];
            k[(size_t)lo * W + q] = k[(size_t)hi * W + q];
            k[(size_t)hi * W + q] = tmp;
          }
          const uint32_t ti = idx[lo];
          idx[lo] = idx[hi];
          idx[hi] = ti;
        }
      }
      __syncthreads();
    }
  }
  // payloads follow their keys: read every original payload before any write
  uint32_t pv[(8192 + kSmallSortThreads - 1) / kSmallSortThreads];
  int u = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) pv[u++] = payload[idx[i]];
  __syncthreads();
  u = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
#pragma unroll
    for (int q = 0; q < W; ++q) keys[(size_t)i * W + q] = k[(size_t)i * W + q];
    payload[i] = pv[u++];
  }
}

}  // namespace edgpu

extern "C" size_t edgpu_sort_states_workspace(int n_words, int64_t n) {
  const int64_t nb = (n + kSortTile - 1) / kSortTile;
  const int64_t hist = 256 * (nb > 0 ? nb : 1);
  size_t bytes = 0;
  bytes += (size_t)n * n_words * sizeof(uint64_t);  // alternate keys
  bytes += (size_t)n * sizeof(uint32_t);            // alternate payload
  bytes = (bytes + 255) & ~(size_t)255;
  bytes += (size_t)hist * sizeof(int64_t);            // histogram
  bytes += (size_t)(hist + 1) * sizeof(int64_t);      // scanned offsets
  bytes += edgpu_scan_workspace(hist);
  return bytes + 512;
}

extern "C" int edgpu_vary_mask(int n_words, const uint64_t* keys, int64_t n, uint64_t* vary_out, void* stream) {
  if (n_words < 1 || n_words > EDGPU_MAX_WORDS || !vary_out || n < 0) return EDGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  cudaMemsetAsync(vary_out, 0, sizeof(uint64_t) * n_words, s);
  if (n == 0) return check_launch();
  EDGPU_DISPATCH_W(n_words, {
    vary_kernel<W><<<grid_for(n, 256), 256, 0, s>>>(keys, n, reinterpret_cast<unsigned long long*>(vary_out)); note_launch();
  });
  return check_launch();
}

extern "C" int edgpu_sort_states(int n_words, uint64_t* keys, uint32_t* payload, int64_t n, const uint64_t* vary_mask,
                                 void* workspace, size_t workspace_bytes, void* stream) {
  if (n_words < 1 || n_words > EDGPU_MAX_WORDS || n < 0) return EDGPU_ERR_ARG;
  if (n <= 1) return EDGPU_OK;
  if (!keys || !payload) return EDGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (small_sort_fits(n_words, n)) {
    const int N = small_sort_pow2(n);
    const size_t smem = (size_t)N * (8 * (size_t)n_words + 4);
    EDGPU_DISPATCH_W(n_words, {
      cudaFuncSetAttribute(small_sort_kernel<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      small_sort_kernel<W><<<1, kSmallSortThreads, smem, s>>>(keys, payload, (int)n, N); note_launch();
    });
    return check_launch();
  }
  if (workspace_bytes < edgpu_sort_states_workspace(n_words, n)) return EDGPU_ERR_WORKSPACE;
  const int64_t nb = (n + kSortTile - 1) / kSortTile;
  const int64_t hist_n = 256 * nb;
  unsigned char* ws = reinterpret_cast<unsigned char*>(workspace);
  size_t off = 0;
  uint64_t* keys_alt = reinterpret_cast<uint64_t*>(ws + off);
  off += (size_t)n * n_words * sizeof(uint64_t);
  uint32_t* pay_alt = reinterpret_cast<uint32_t*>(ws + off);
  off += (size_t)n * sizeof(uint32_t);
  off = (off + 255) & ~(size_t)255;
  int64_t* hist = reinterpret_cast<int64_t*>(ws + off);
  off += (size_t)hist_n * sizeof(int64_t);
  int64_t* offs = reinterpret_cast<int64_t*>(ws + off);
  off += (size_t)(hist_n + 1) * sizeof(int64_t);
  void* scan_ws = ws + off;
  const size_t scan_bytes = workspace_bytes - off;

  uint64_t* kin = keys;
  uint32_t* pin = payload;
  uint64_t* kout = keys_alt;
  uint32_t* pout = pay_alt;
  int rc = EDGPU_OK;
  for (int q = n_words - 1; q >= 0; --q) {
    for (int byte = 0; byte < 8; ++byte) {
      const int shift = 8 * byte;
      if (vary_mask && ((vary_mask[q] >> shift) & 0xFFull) == 0) continue;
      EDGPU_DISPATCH_W(n_words, {
        radix_hist_kernel<W><<<(unsigned)nb, kSortThreads, 0, s>>>(kin, n, q, shift, hist, nb); note_launch();
      });
      if ((rc = check_launch())) return rc;
      if ((rc = edgpu_scan_i64(hist, offs, hist_n, scan_ws, scan_bytes, stream))) return rc;
      EDGPU_DISPATCH_W(n_words, {
        radix_scatter_kernel<W><<<(unsigned)nb, kSortThreads, 0, s>>>(kin, pin, kout, pout, n, q, shift, offs, nb); note_launch();
      });
      if ((rc = check_launch())) return rc;
      uint64_t* tk = kin;
      kin = kout;
      kout = tk;
      uint32_t* tp = pin;
      pin = pout;
      pout = tp;
    }
  }
  if (kin != keys) {
    EDGPU_DISPATCH_W(n_words, { copy_states_kernel<W><<<grid_for(n, 256), 256, 0, s>>>(kin, pin, keys, payload, n); note_launch(); });
    rc = check_launch();
  }
  return rc;
}

extern "C" int edgpu_segment_heads(int n_words, const uint64_t* keys, int64_t n, int64_t* head, void* stream) {
  if (n < 0 || (n > 0 && (!keys || !head))) return EDGPU_ERR_ARG;
  if (n == 0) return EDGPU_OK;
  EDGPU_DISPATCH_W(n_words, { heads_kernel<W><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(keys, n, head); note_launch(); });
  return check_launch();
}

extern "C" int edgpu_segment_reduce(int n_words, const uint64_t* keys, const uint32_t* payload, int64_t n,
                                    const int64_t* head_scan, const double* vals, uint64_t* out_keys,
                                    uint32_t* out_first, double* out_vals, void* stream) {
  if (n < 0 || (n > 0 && (!keys || !payload || !head_scan || !out_keys))) return EDGPU_ERR_ARG;
  if (n == 0) return EDGPU_OK;
  EDGPU_DISPATCH_W(n_words, {
    segment_reduce_kernel<W><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        keys, payload, n, head_scan, reinterpret_cast<const double2*>(vals), out_keys, out_first,
        reinterpret_cast<double2*>(out_vals)); note_launch();
  });
  return check_launch();
}

extern "C" int edgpu_merge_states(int n_words, const uint64_t* a, int64_t na, const uint64_t* b, int64_t nb,
                                  uint64_t* out, void* stream) {
  if (na < 0 || nb < 0 || !out) return EDGPU_ERR_ARG;
  if (na + nb == 0) return EDGPU_OK;
  EDGPU_DISPATCH_W(n_words, {
    merge_kernel<W><<<grid_for(na + nb, 256), 256, 0, (cudaStream_t)stream>>>(a, na, b, nb, out); note_launch();
  });
  return check_launch();
}

extern "C" int edgpu_lookup_states(int n_words, const uint64_t* basis, int64_t n_basis, const uint64_t* query,
                                   int64_t nq, int64_t* out_index, void* stream) {
  if (nq < 0 || n_basis < 0 || (nq > 0 && (!query || !out_index))) return EDGPU_ERR_ARG;
  if (nq == 0) return EDGPU_OK;
  EDGPU_DISPATCH_W(n_words, {
    lookup_kernel<W><<<grid_for(nq, 256), 256, 0, (cudaStream_t)stream>>>(basis, n_basis, query, nq, out_index); note_launch();
  });
  return check_launch();
}
