// H·v for R vectors with a row schedule (edgpu_spmv_plan, edgpu_spmv_planned[_c64]).
//
// y[i][0..R) = sum_e H[i][col[e]] x[col[e]][0..R), the vectors stored run-fastest, so one row
// of x is R complex numbers = L 16-byte packs (L = R / runs-per-pack).  A group of L lanes
// serves one row: lane q gathers pack q of every x row the row's entries name, so each
// gather of a group is one contiguous x row (for R = 16 complex64: one 128-byte line).
//
// The cost of the kernel is the gathers of x rows from L2 (nnz of them; x itself is read
// from HBM once): on the 462 120-state photoemission sector of the 316-spin-orbital model
// (4.7 M entries, R = 16 complex64) they move 604 MB from L2 to the SMs per launch.  What
// limits a row-per-group kernel there is not L2 bandwidth but (a) warps whose groups hold
// rows of different lengths (the group with the longest row sets the warp's time) and
// (b) the chain of dependent gather batches of the longest rows (up to ~200 entries).  The
// schedule removes both:
//   * heavy rows (length >= heavy_min) come first, longest first, one warp per row: the
//     32 / L groups of the warp take every (32 / L)-th entry and the partial sums are added
//     across the groups with xor shuffles in a fixed order;
//   * the other rows follow, sorted by length (longest first) within windows of `window`
//     consecutive rows, so the 32 / L rows a warp serves together have nearly equal lengths
//     while the rows of a window stay together (their x rows overlap: L1 reuse).
// Each lane keeps U gathers in flight per batch (predicated tail, no divergence inside a
// group).  The plan (the schedule and the count of heavy rows) is built once per matrix by a
// stable radix sort of one 64-bit key per row.
#include "common.cuh"

namespace edgpu {
namespace {

template <typename T>
struct Pack16;
template <>
struct Pack16<float> {
  using type = float4;
  static constexpr int runs = 2;
};
template <>
struct Pack16<double> {
  using type = double2;
  static constexpr int runs = 1;
};

template <typename T, bool VALC, int L, int U>
__global__ void spmv_sched_kernel(int64_t n_heavy, int64_t n, const int64_t* __restrict__ rp,
                                  const int32_t* __restrict__ col, const T* __restrict__ vals,
                                  const int32_t* __restrict__ sched, const typename Pack16<T>::type* __restrict__ X,
                                  typename Pack16<T>::type* __restrict__ Y) {
  using P = typename Pack16<T>::type;
  constexpr int RV = Pack16<T>::runs;
  constexpr int G = 32 / L;  // row groups per warp
  const int lane = threadIdx.x & 31;
  const int grp = lane / L, sub = lane - grp * L;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const bool heavy = warp < n_heavy;  // warp-uniform
  int64_t row = -1, e = 0, e1 = 0;
  int stride = 1;
  if (heavy) {
    row = __ldg(sched + warp);
    e = __ldg(rp + row) + grp;
    e1 = __ldg(rp + row + 1);
    stride = G;
  } else {
    const int64_t k = n_heavy + (warp - n_heavy) * G + grp;
    if (k < n) {
      row = __ldg(sched + k);
      e = __ldg(rp + row);
      e1 = __ldg(rp + row + 1);
    }
  }
  T ar[RV], ai[RV];
#pragma unroll
  for (int q = 0; q < RV; ++q) ar[q] = ai[q] = T(0);
  for (; e < e1; e += (int64_t)stride * U) {
    int c[U];
    T hr[U], hi[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t eu = e + (int64_t)u * stride;
      const bool ok = eu < e1;
      // the CSR is read once: streaming loads leave L2 to x
      c[u] = ok ? __ldcs(col + eu) : 0;
      if (VALC) {
        hr[u] = ok ? __ldcs(vals + 2 * eu) : T(0);
        hi[u] = ok ? __ldcs(vals + 2 * eu + 1) : T(0);
      } else {
        hr[u] = ok ? __ldcs(vals + eu) : T(0);
        hi[u] = T(0);
      }
    }
    P xv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) xv[u] = (e + (int64_t)u * stride < e1) ? __ldg(X + (int64_t)c[u] * L + sub) : P{};
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const T* xs = reinterpret_cast<const T*>(&xv[u]);
#pragma unroll
      for (int q = 0; q < RV; ++q) {
        const T xr = xs[2 * q], xi = xs[2 * q + 1];
        ar[q] += hr[u] * xr;
        ai[q] += hr[u] * xi;
        if (VALC) {
          ar[q] -= hi[u] * xi;
          ai[q] += hi[u] * xr;
        }
      }
    }
  }
  if (heavy) {
#pragma unroll
    for (int o = L; o < 32; o <<= 1)
#pragma unroll
      for (int q = 0; q < RV; ++q) {
        ar[q] += __shfl_xor_sync(0xffffffffu, ar[q], o);
        ai[q] += __shfl_xor_sync(0xffffffffu, ai[q], o);
      }
    if (grp != 0) return;
  }
  if (row < 0) return;
  P out;
  T* os = reinterpret_cast<T*>(&out);
#pragma unroll
  for (int q = 0; q < RV; ++q) {
    os[2 * q] = ar[q];
    os[2 * q + 1] = ai[q];
  }
  __stcs(Y + row * L + sub, out);
}

// One key per row: bit 63 set for light rows (heavy rows sort first), bits 39..62 the
// window of a light row, bits 19..38 the inverted length (longest first).
__global__ void spmv_plan_keys_kernel(int64_t n, const int64_t* __restrict__ rp, int64_t window, int heavy_min,
                                      uint64_t* keys, uint32_t* payload, unsigned long long* n_heavy) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t len = rp[i + 1] - rp[i];
  const bool light = len < heavy_min;
  const uint64_t inv = (uint64_t)(0xFFFFF - (len < 0xFFFFF ? len : 0xFFFFF));
  uint64_t key = (inv << 19);
  if (light) key |= (1ull << 63) | ((uint64_t)(i / window) << 39);
  keys[i] = key;
  payload[i] = (uint32_t)i;
  if (!light) atomicAdd(n_heavy, 1ull);
}

template <typename T, bool VALC, int L>
int launch_sched(const edgpu_csr* h, const T* vals, const int32_t* sched, int64_t n_heavy, int unroll, int block,
                 const void* x, void* y, cudaStream_t s) {
  using P = typename Pack16<T>::type;
  constexpr int G = 32 / L;
  const int64_t n = h->n;
  const int64_t warps = n_heavy + (n - n_heavy + G - 1) / G;
  const int64_t blocks = (warps * 32 + block - 1) / block;
  if (blocks > 0x7fffffffLL) return EDGPU_ERR_ARG;
  const P* X = reinterpret_cast<const P*>(x);
  P* Y = reinterpret_cast<P*>(y);
  if (unroll == 4)
    spmv_sched_kernel<T, VALC, L, 4><<<(unsigned)blocks, block, 0, s>>>(n_heavy, n, h->row_ptr, h->col, vals, sched,
                                                                        X, Y);
  else if (unroll == 8)
    spmv_sched_kernel<T, VALC, L, 8><<<(unsigned)blocks, block, 0, s>>>(n_heavy, n, h->row_ptr, h->col, vals, sched,
                                                                        X, Y);
  else
    spmv_sched_kernel<T, VALC, L, 2><<<(unsigned)blocks, block, 0, s>>>(n_heavy, n, h->row_ptr, h->col, vals, sched,
                                                                        X, Y);
  note_launch();
  return check_launch();
}

template <typename T, bool VALC>
int dispatch_lanes(const edgpu_csr* h, const T* vals, const int32_t* sched, int64_t n_heavy, int unroll, int block,
                   const void* x, void* y, int L, cudaStream_t s) {
  switch (L) {
    case 1: return launch_sched<T, VALC, 1>(h, vals, sched, n_heavy, unroll, block, x, y, s);
    case 2: return launch_sched<T, VALC, 2>(h, vals, sched, n_heavy, unroll, block, x, y, s);
    case 4: return launch_sched<T, VALC, 4>(h, vals, sched, n_heavy, unroll, block, x, y, s);
    case 8: return launch_sched<T, VALC, 8>(h, vals, sched, n_heavy, unroll, block, x, y, s);
    case 16: return launch_sched<T, VALC, 16>(h, vals, sched, n_heavy, unroll, block, x, y, s);
    case 32: return launch_sched<T, VALC, 32>(h, vals, sched, n_heavy, unroll, block, x, y, s);
    default: return EDGPU_ERR_ARG;
  }
}

template <typename T>
int spmv_planned(const edgpu_csr* h, const int32_t* sched, int64_t n_heavy, int unroll, int block, const void* x,
                 void* y, int R, const T* val_c, const T* val_r, cudaStream_t s) {
  if (!h || !sched || !x || !y || h->n < 1 || R < 1) return EDGPU_ERR_ARG;
  if (n_heavy < 0 || n_heavy > h->n) return EDGPU_ERR_ARG;
  if (unroll != 2 && unroll != 4 && unroll != 8) return EDGPU_ERR_ARG;
  if (block != 64 && block != 128 && block != 256 && block != 512) return EDGPU_ERR_ARG;
  constexpr int RV = Pack16<T>::runs;
  if (R % RV) return EDGPU_ERR_ARG;
  const int L = R / RV;
  if (L > 32 || (32 % L)) return EDGPU_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15) return EDGPU_ERR_ARG;
  if (val_c) return dispatch_lanes<T, true>(h, val_c, sched, n_heavy, unroll, block, x, y, L, s);
  if (val_r) return dispatch_lanes<T, false>(h, val_r, sched, n_heavy, unroll, block, x, y, L, s);
  return EDGPU_ERR_ARG;
}

}  // namespace
}  // namespace edgpu

using namespace edgpu;

extern "C" size_t edgpu_spmv_plan_workspace(int64_t n) {
  if (n < 1) return 0;
  return edgpu_sort_states_workspace(1, n) + 8 * (size_t)n + 1024;
}

extern "C" int edgpu_spmv_plan(const edgpu_csr* h, int64_t window, int heavy_min, int32_t* sched, int64_t* n_heavy,
                               void* workspace, size_t workspace_bytes, void* stream) {
  if (!h || !sched || !n_heavy || h->n < 1 || !h->row_ptr) return EDGPU_ERR_ARG;
  if (heavy_min < 1 || window < 0) return EDGPU_ERR_ARG;
  const int64_t n = h->n;
  if (n >= (1ll << 31)) return EDGPU_ERR_ARG;
  if (window == 0 || window > n) window = n;
  const int64_t n_win = (n + window - 1) / window;
  if (n_win >= (1ll << 24)) return EDGPU_ERR_ARG;
  if (workspace_bytes < edgpu_spmv_plan_workspace(n)) return EDGPU_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char* ws = reinterpret_cast<unsigned char*>(workspace);
  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(ws);
  uint64_t* keys = reinterpret_cast<uint64_t*>(ws + 256);
  unsigned char* sort_ws = ws + 256 + ((8 * (size_t)n + 255) & ~(size_t)255);
  const size_t sort_bytes = workspace_bytes - (size_t)(sort_ws - ws);
  if (cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s) != cudaSuccess) return EDGPU_ERR_CUDA;
  spmv_plan_keys_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, h->row_ptr, window, heavy_min, keys,
                                                                    reinterpret_cast<uint32_t*>(sched), cnt);
  note_launch();
  int rc = check_launch();
  if (rc) return rc;
  // bits that can differ between keys: the light flag, the window number, the length
  uint64_t wbits = 1;
  while ((int64_t)wbits < n_win) wbits <<= 1;
  const uint64_t vary = (1ull << 63) | ((wbits - 1) << 39) | (0xFFFFFull << 19);
  rc = edgpu_sort_states(1, keys, reinterpret_cast<uint32_t*>(sched), n, &vary, sort_ws, sort_bytes, stream);
  if (rc) return rc;
  unsigned long long nh = 0;
  if (cudaMemcpyAsync(&nh, cnt, sizeof(nh), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return EDGPU_ERR_CUDA;
  *n_heavy = (int64_t)nh;
  return EDGPU_OK;
}

extern "C" int edgpu_spmv_planned(const edgpu_csr* h, const int32_t* sched, int64_t n_heavy, int unroll, int block,
                                  const double* x, double* y, int R, void* stream) {
  if (!h) return EDGPU_ERR_ARG;
  return spmv_planned<double>(h, sched, n_heavy, unroll, block, x, y, R, h->val_c, h->val_r, (cudaStream_t)stream);
}

extern "C" int edgpu_spmv_planned_c64(const edgpu_csr* h, const int32_t* sched, int64_t n_heavy, int unroll,
                                      int block, const float* x, float* y, int R, void* stream) {
  if (!h) return EDGPU_ERR_ARG;
  return spmv_planned<float>(h, sched, n_heavy, unroll, block, x, y, R, h->val_cf, h->val_rf, (cudaStream_t)stream);
}
