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
#include <climits>
#include <vector>

#include "common.cuh"
#include "pages.cuh"

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
                 const void* x, void* y, cudaStream_t s, int64_t n_rows = -1) {
  using P = typename Pack16<T>::type;
  constexpr int G = 32 / L;
  const int64_t n = n_rows < 0 ? h->n : n_rows;  // n_rows = n_heavy: the heavy rows only
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
                   const void* x, void* y, int L, cudaStream_t s, int64_t n_rows = -1) {
  switch (L) {
    case 1: return launch_sched<T, VALC, 1>(h, vals, sched, n_heavy, unroll, block, x, y, s, n_rows);
    case 2: return launch_sched<T, VALC, 2>(h, vals, sched, n_heavy, unroll, block, x, y, s, n_rows);
    case 4: return launch_sched<T, VALC, 4>(h, vals, sched, n_heavy, unroll, block, x, y, s, n_rows);
    case 8: return launch_sched<T, VALC, 8>(h, vals, sched, n_heavy, unroll, block, x, y, s, n_rows);
    case 16: return launch_sched<T, VALC, 16>(h, vals, sched, n_heavy, unroll, block, x, y, s, n_rows);
    case 32: return launch_sched<T, VALC, 32>(h, vals, sched, n_heavy, unroll, block, x, y, s, n_rows);
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


// ---------------------------------------------------------------------------------------
// Paged layout (edgpu_spmv_pages_build / edgpu_spmv_paged[_c64]).
//
// The rows of a schedule are cut into slices and packed whole, in schedule order, into
// fixed-size pages of CH entries.  A heavy row is a slice of its own whose entries are dealt
// to the C = 32 / L row groups of a warp in turn (group r takes entries r, r + C, ...); a
// light slice holds C consecutive light rows, one per group.  A page is a header column (C
// entries; the first holds the number of used columns), then per slice a header column
// (entry r: column -2 - row of group r, or INT_MIN for none, and a flag set for a heavy row)
// and the slice's entry columns (entry (k, r): column and value of the group's k-th entry,
// column -1 past its end).
//
// One warp serves one page: it copies the page into shared memory with cp.async (16-byte
// chunks, coalesced) and reads its columns as one stream, U columns per batch, so U gathers
// of x rows per lane are in flight whatever the slice boundaries; a slice header column
// closes the groups' previous rows (adding a heavy row's partial sums across the groups with
// xor shuffles) and opens the next.  The only memory latencies on a warp's path are the page
// copy and the gathers; the rows, columns and values come from shared memory.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16_hint(void* smem, const void* gmem, uint64_t pol) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// L2 eviction-priority policies (PTX createpolicy): x rows are gathered nnz times and should
// stay in L2; pages are read once.
__device__ __forceinline__ uint64_t l2_policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;\n" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(p));
  return p;
}
__device__ __forceinline__ float4 ldg_hint(const float4* ptr, uint64_t pol) {
  float4 v;
  asm volatile("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;\n"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(ptr), "l"(pol));
  return v;
}
__device__ __forceinline__ double2 ldg_hint(const double2* ptr, uint64_t pol) {
  double2 v;
  asm volatile("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;\n" : "=d"(v.x), "=d"(v.y) : "l"(ptr), "l"(pol));
  return v;
}

constexpr int kPageWarps = 4;  // warps (pages) per block of the paged kernel

template <typename T, bool VALC, int L, int U, int CH, bool PIPE, bool HINT>
__global__ void __launch_bounds__(32 * kPageWarps) spmv_pages_kernel(int64_t n_pages,
                                                                     const Ent<T, VALC>* __restrict__ pages,
                                                                     const typename Pack16<T>::type* __restrict__ X,
                                                                     typename Pack16<T>::type* __restrict__ Y) {
  using E = Ent<T, VALC>;
  using P = typename Pack16<T>::type;
  constexpr int RV = Pack16<T>::runs;
  constexpr int C = 32 / L;
  constexpr int CHUNKS = CH * (int)sizeof(E) / 16;  // 16-byte copies per page
  extern __shared__ __align__(16) unsigned char page_raw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int grp = lane / L, sub = lane - grp * L;
  const int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (p >= n_pages) return;  // warp-uniform
  E* pg = reinterpret_cast<E*>(page_raw) + (size_t)wib * CH;
  uint64_t pol_x = 0;
  {
    const unsigned char* src = reinterpret_cast<const unsigned char*>(pages + p * CH);
    unsigned char* dst = reinterpret_cast<unsigned char*>(pg);
    if constexpr (HINT) {
      pol_x = l2_policy_evict_last();
      const uint64_t pol_p = l2_policy_evict_first();
#pragma unroll
      for (int k = lane; k < CHUNKS; k += 32) cp_async16_hint(dst + 16 * k, src + 16 * k, pol_p);
    } else {
#pragma unroll
      for (int k = lane; k < CHUNKS; k += 32) cp_async16(dst + 16 * k, src + 16 * k);
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncwarp();
  }
  T ar[RV], ai[RV];
#pragma unroll
  for (int q = 0; q < RV; ++q) ar[q] = ai[q] = T(0);
  int64_t row = -1;
  bool heavy = false;
  auto flush = [&]() {  // called by the whole warp at the same column
    if (heavy) {
#pragma unroll
      for (int o = L; o < 32; o <<= 1)
#pragma unroll
        for (int q = 0; q < RV; ++q) {
          ar[q] += __shfl_xor_sync(0xffffffffu, ar[q], o);
          ai[q] += __shfl_xor_sync(0xffffffffu, ai[q], o);
        }
    }
    if (row >= 0 && (!heavy || grp == 0)) {
      P out;
      T* os = reinterpret_cast<T*>(&out);
#pragma unroll
      for (int q = 0; q < RV; ++q) {
        os[2 * q] = ar[q];
        os[2 * q + 1] = ai[q];
      }
      __stcs(Y + row * L + sub, out);
    }
#pragma unroll
    for (int q = 0; q < RV; ++q) ar[q] = ai[q] = T(0);
  };
  const int ncols = pg[0].c;
  E en[U];
  P xv[U];
  // batch k: U columns from shared memory, then their gathers (issued before the previous
  // batch is consumed when PIPE, so two batches of gathers are in flight)
  auto fetch = [&](int k, E* e, P* x) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (k + u < ncols) {
        e[u] = pg[(k + u) * C + grp];
      } else {
        e[u] = E{};
        e[u].c = -1;
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if constexpr (HINT) {
        x[u] = e[u].c >= 0 ? ldg_hint(X + (int64_t)e[u].c * L + sub, pol_x) : P{};
      } else {
        x[u] = e[u].c >= 0 ? __ldg(X + (int64_t)e[u].c * L + sub) : P{};
      }
    }
  };
  auto consume = [&](const E* e, const P* x) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int c = e[u].c;
      if (c <= -2) {  // a slice header column (the same kind in every group)
        flush();
        row = c == INT_MIN ? -1 : (int64_t)(-2 - (int64_t)c);
        heavy = e[u].flag() != 0;
        continue;
      }
      if (c < 0) continue;
      const T* xs = reinterpret_cast<const T*>(&x[u]);
      T hr, hi = T(0);
      if constexpr (VALC) {
        hr = e[u].vr;
        hi = e[u].vi;
      } else {
        hr = e[u].v;
      }
#pragma unroll
      for (int q = 0; q < RV; ++q) {
        const T xr = xs[2 * q], xi = xs[2 * q + 1];
        ar[q] += hr * xr;
        ai[q] += hr * xi;
        if (VALC) {
          ar[q] -= hi * xi;
          ai[q] += hi * xr;
        }
      }
    }
  };
  if constexpr (PIPE) {
    E en2[U];
    P xv2[U];
    if (1 < ncols) fetch(1, en, xv);
    for (int k = 1; k < ncols; k += 2 * U) {
      if (k + U < ncols) fetch(k + U, en2, xv2);
      consume(en, xv);
      if (k + U >= ncols) break;
      if (k + 2 * U < ncols) fetch(k + 2 * U, en, xv);
      consume(en2, xv2);
    }
  } else {
    for (int k = 1; k < ncols; k += U) {
      fetch(k, en, xv);
      consume(en, xv);
    }
  }
  flush();
}

// Slice widths: heavy slice s < n_heavy: ceil(len / C); light slices: the longest row.
__global__ void pages_width_kernel(int64_t n_heavy, int64_t n_rows, int64_t n_slices, int C,
                                   const int32_t* __restrict__ sched, const int64_t* __restrict__ rp,
                                   int32_t* wout) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_slices) return;
  int64_t w = 0;
  if (s < n_heavy) {
    const int64_t row = sched[s];
    w = (rp[row + 1] - rp[row] + C - 1) / C;
  } else {
    for (int r = 0; r < C; ++r) {
      const int64_t q = n_heavy + (s - n_heavy) * C + r;
      if (q < n_rows) {
        const int64_t row = sched[q];
        const int64_t len = rp[row + 1] - rp[row];
        w = len > w ? len : w;
      }
    }
  }
  wout[s] = (int32_t)w;
}

template <typename E>
__device__ __forceinline__ E make_ent(int32_t c, int flag) {
  E e{};
  e.c = c;
  e.set_flag(flag);
  return e;
}

// Every entry of every page: empty (column -1, value 0); the first header entry of a page:
// its number of used columns.
template <typename E>
__global__ void pages_clear_kernel(int64_t n_pages, int CH, const int32_t* __restrict__ page_cols, E* pages) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pages * CH) return;
  const int64_t p = i / CH;
  const int k = (int)(i - p * CH);
  pages[i] = make_ent<E>(k == 0 ? page_cols[p] : -1, 0);
}

// One warp per slice: its header column and w entry columns at its place in its page.
template <typename T, bool VALC>
__global__ void pages_fill_kernel(int64_t n_slices, int64_t n_heavy, int64_t n_rows, int C,
                                  const int32_t* __restrict__ sched, const int64_t* __restrict__ rp,
                                  const int32_t* __restrict__ col, const T* __restrict__ vals,
                                  const int32_t* __restrict__ width, const int64_t* __restrict__ slice_pos,
                                  Ent<T, VALC>* pages) {
  using E = Ent<T, VALC>;
  const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (s >= n_slices) return;
  const int w = width[s];
  const bool hv = s < n_heavy;
  E* base = pages + slice_pos[s];
  for (int k = lane; k < (w + 1) * C; k += 32) {
    const int e = k / C - 1, r = k - (k / C) * C;
    int64_t row, idx;
    if (hv) {
      row = sched[s];
      idx = (int64_t)e * C + r;  // heavy row: entries dealt to the groups in turn
    } else {
      const int64_t q = n_heavy + (s - n_heavy) * C + r;
      row = q < n_rows ? sched[q] : -1;
      idx = e;
    }
    if (e < 0) {
      base[k] = make_ent<E>(row >= 0 ? (int32_t)(-2 - row) : INT_MIN, hv ? 1 : 0);
      continue;
    }
    E en = make_ent<E>(-1, 0);
    if (row >= 0) {
      const int64_t e0 = rp[row], len = rp[row + 1] - e0;
      if (idx < len) {
        en.c = col[e0 + idx];
        if constexpr (VALC) {
          en.vr = vals[2 * (e0 + idx)];
          en.vi = vals[2 * (e0 + idx) + 1];
        } else {
          en.v = vals[e0 + idx];
        }
      }
    }
    base[k] = en;
  }
}

template <typename T, bool VALC, int L, int U, int CH>
int launch_pages_t(int64_t n_pages, const void* pages, const void* x, void* y, cudaStream_t s, int flags) {
  using P = typename Pack16<T>::type;
  using E = Ent<T, VALC>;
  auto kern = (flags & 1) ? ((flags & 2) ? spmv_pages_kernel<T, VALC, L, U, CH, true, true>
                                         : spmv_pages_kernel<T, VALC, L, U, CH, true, false>)
                          : ((flags & 2) ? spmv_pages_kernel<T, VALC, L, U, CH, false, true>
                                         : spmv_pages_kernel<T, VALC, L, U, CH, false, false>);
  const size_t smem = (size_t)kPageWarps * CH * sizeof(E);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return EDGPU_ERR_CUDA;
  }
  const int64_t blocks = (n_pages + kPageWarps - 1) / kPageWarps;
  if (blocks > 0x7fffffffLL) return EDGPU_ERR_ARG;
  kern<<<(unsigned)blocks, 32 * kPageWarps, smem, s>>>(n_pages, reinterpret_cast<const E*>(pages),
                                                        reinterpret_cast<const P*>(x), reinterpret_cast<P*>(y));
  note_launch();
  return check_launch();
}

// unroll: 4 or 8 gathers per lane per batch; flags bit 0: two batches in flight, bit 1: L2
// eviction hints (x rows evict-last, pages evict-first)
template <typename T, bool VALC, int L>
int launch_pages_l(int64_t n_pages, const void* pages, int CH, int unroll, int flags, const void* x, void* y,
                   cudaStream_t s) {
  if (CH == 256 && unroll == 4) return launch_pages_t<T, VALC, L, 4, 256>(n_pages, pages, x, y, s, flags);
  if (CH == 256 && unroll == 8) return launch_pages_t<T, VALC, L, 8, 256>(n_pages, pages, x, y, s, flags);
  if (CH == 512 && unroll == 4) return launch_pages_t<T, VALC, L, 4, 512>(n_pages, pages, x, y, s, flags);
  if (CH == 512 && unroll == 8) return launch_pages_t<T, VALC, L, 8, 512>(n_pages, pages, x, y, s, flags);
  if (CH == 1024 && unroll == 4) return launch_pages_t<T, VALC, L, 4, 1024>(n_pages, pages, x, y, s, flags);
  if (CH == 1024 && unroll == 8) return launch_pages_t<T, VALC, L, 8, 1024>(n_pages, pages, x, y, s, flags);
  return EDGPU_ERR_ARG;
}

template <typename T, bool VALC>
int launch_pages(int64_t n_pages, const void* pages, int CH, int unroll, int flags, int L, const void* x, void* y,
                 cudaStream_t s) {
  switch (L) {
    case 2: return launch_pages_l<T, VALC, 2>(n_pages, pages, CH, unroll, flags, x, y, s);
    case 4: return launch_pages_l<T, VALC, 4>(n_pages, pages, CH, unroll, flags, x, y, s);
    case 8: return launch_pages_l<T, VALC, 8>(n_pages, pages, CH, unroll, flags, x, y, s);
    case 16: return launch_pages_l<T, VALC, 16>(n_pages, pages, CH, unroll, flags, x, y, s);
    default: return EDGPU_ERR_ARG;
  }
}

// value kinds of the paged layout (entry sizes 8, 16, 16 bytes)
enum { kPagesRealF = 0, kPagesRealD = 1, kPagesCplxF = 2 };

template <typename T, bool VALC>
int fill_pages(const edgpu_csr* h, const T* vals, const int32_t* sched, int64_t n_heavy, int C, int CH,
               const int32_t* width, const int64_t* slice_pos, const int32_t* page_cols, int64_t n_slices,
               int64_t n_pages, void* pages, cudaStream_t s) {
  using E = Ent<T, VALC>;
  const int64_t total = n_pages * CH;
  pages_clear_kernel<E><<<(unsigned)((total + 255) / 256), 256, 0, s>>>(n_pages, CH, page_cols,
                                                                        reinterpret_cast<E*>(pages));
  note_launch();
  pages_fill_kernel<T, VALC><<<(unsigned)((n_slices * 32 + 255) / 256), 256, 0, s>>>(
      n_slices, n_heavy, h->n, C, sched, h->row_ptr, h->col, vals, width, slice_pos, reinterpret_cast<E*>(pages));
  note_launch();
  return check_launch();
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

extern "C" size_t edgpu_spmv_pages_workspace(int64_t n, int lanes) {
  if (n < 1 || lanes < 1 || lanes > 32) return 0;
  const int64_t n_slices = n;  // at most one slice per row
  return 256 + ((sizeof(int32_t) * (size_t)n_slices + 255) & ~(size_t)255) +
         ((sizeof(int64_t) * (size_t)n_slices + 255) & ~(size_t)255) + sizeof(int32_t) * (size_t)(n_slices + 2);
}

extern "C" int edgpu_spmv_pages_build(const edgpu_csr* h, const int32_t* sched, int64_t n_heavy, int lanes,
                                      int page_entries, int value_kind, void* pages, int64_t cap_pages,
                                      int64_t* n_pages, void* workspace, size_t workspace_bytes, void* stream) {
  if (!h || !sched || !n_pages || h->n < 1 || n_heavy < 0 || n_heavy > h->n) return EDGPU_ERR_ARG;
  if (h->n >= (1ll << 31) - 2) return EDGPU_ERR_ARG;
  if (lanes != 2 && lanes != 4 && lanes != 8 && lanes != 16) return EDGPU_ERR_ARG;
  if (page_entries != 256 && page_entries != 512 && page_entries != 1024) return EDGPU_ERR_ARG;
  const void* vals = value_kind == kPagesRealF ? (const void*)h->val_rf
                     : value_kind == kPagesRealD ? (const void*)h->val_r
                     : value_kind == kPagesCplxF ? (const void*)h->val_cf : nullptr;
  if (!vals) return EDGPU_ERR_ARG;
  if (workspace_bytes < edgpu_spmv_pages_workspace(h->n, lanes)) return EDGPU_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const int C = 32 / lanes, CH = page_entries;
  const int64_t n_light = h->n - n_heavy, n_slices = n_heavy + (n_light + C - 1) / C;
  unsigned char* ws = reinterpret_cast<unsigned char*>(workspace);
  int32_t* width = reinterpret_cast<int32_t*>(ws + 256);
  int64_t* slice_pos = reinterpret_cast<int64_t*>(ws + 256 + ((sizeof(int32_t) * (size_t)h->n + 255) & ~(size_t)255));
  int32_t* page_cols = reinterpret_cast<int32_t*>(reinterpret_cast<unsigned char*>(slice_pos) +
                                                  ((sizeof(int64_t) * (size_t)h->n + 255) & ~(size_t)255));
  std::vector<int32_t> w_h((size_t)n_slices);
  if (n_slices > 0) {
    pages_width_kernel<<<(unsigned)((n_slices + 255) / 256), 256, 0, s>>>(n_heavy, h->n, n_slices, C, sched,
                                                                          h->row_ptr, width);
    note_launch();
    if (check_launch() != EDGPU_OK ||
        cudaMemcpyAsync(w_h.data(), width, sizeof(int32_t) * (size_t)n_slices, cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return EDGPU_ERR_CUDA;
  }
  // greedy packing in schedule order: a page holds its header column and whole slices
  std::vector<int64_t> pos_h((size_t)n_slices);
  std::vector<int32_t> cols_h;  // used columns of each page (its header column included)
  int64_t page = 0, used = C;
  for (int64_t sl = 0; sl < n_slices; ++sl) {
    const int64_t size = (int64_t)C * (w_h[(size_t)sl] + 1);
    if (size + C > CH) return EDGPU_ERR_ARG;  // a row too long for the page size
    if (used + size > CH) {
      cols_h.push_back((int32_t)(used / C));
      ++page;
      used = C;
    }
    pos_h[(size_t)sl] = page * CH + used;
    used += size;
  }
  cols_h.push_back((int32_t)(used / C));
  const int64_t np = n_slices > 0 ? page + 1 : 0;
  *n_pages = np;
  if (np > cap_pages || (np > 0 && !pages)) return EDGPU_ERR_OVERFLOW;
  if (np == 0) return EDGPU_OK;
  if ((reinterpret_cast<uintptr_t>(pages) & 15) != 0) return EDGPU_ERR_ARG;
  if (cudaMemcpyAsync(slice_pos, pos_h.data(), sizeof(int64_t) * (size_t)n_slices, cudaMemcpyHostToDevice, s) !=
          cudaSuccess ||
      cudaMemcpyAsync(page_cols, cols_h.data(), sizeof(int32_t) * (size_t)np, cudaMemcpyHostToDevice, s) !=
          cudaSuccess)
    return EDGPU_ERR_CUDA;
  int rc;
  if (value_kind == kPagesRealF)
    rc = fill_pages<float, false>(h, h->val_rf, sched, n_heavy, C, CH, width, slice_pos, page_cols, n_slices, np,
                                  pages, s);
  else if (value_kind == kPagesRealD)
    rc = fill_pages<double, false>(h, h->val_r, sched, n_heavy, C, CH, width, slice_pos, page_cols, n_slices, np,
                                   pages, s);
  else
    rc = fill_pages<float, true>(h, h->val_cf, sched, n_heavy, C, CH, width, slice_pos, page_cols, n_slices, np,
                                 pages, s);
  if (rc) return rc;
  // the host vectors above are read by the copies: wait for them before they go out of scope
  return cudaStreamSynchronize(s) == cudaSuccess ? EDGPU_OK : EDGPU_ERR_CUDA;
}

template <typename T>
static int spmv_paged_impl(const edgpu_csr* h, const void* pages, int64_t n_pages, int page_entries, int unroll,
                           int flags, const void* x, void* y, int R, cudaStream_t s) {
  if (!h || !x || !y || h->n < 1 || n_pages < 0) return EDGPU_ERR_ARG;
  if (n_pages > 0 && !pages) return EDGPU_ERR_ARG;
  if ((unroll != 4 && unroll != 8) || flags < 0 || flags > 3) return EDGPU_ERR_ARG;
  constexpr int RV = Pack16<T>::runs;
  if (R % RV) return EDGPU_ERR_ARG;
  const int L = R / RV;
  if (L != 2 && L != 4 && L != 8 && L != 16) return EDGPU_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y) | reinterpret_cast<uintptr_t>(pages)) & 15)
    return EDGPU_ERR_ARG;
  if (sizeof(T) == 8 && (h->val_c || !h->val_r)) return EDGPU_ERR_ARG;  // complex128 values: no paged form
  if (sizeof(T) == 4 && !h->val_cf && !h->val_rf) return EDGPU_ERR_ARG;
  if (n_pages == 0) return EDGPU_OK;
  if (sizeof(T) == 8) return launch_pages<double, false>(n_pages, pages, page_entries, unroll, flags, L, x, y, s);
  if (h->val_cf) return launch_pages<float, true>(n_pages, pages, page_entries, unroll, flags, L, x, y, s);
  return launch_pages<float, false>(n_pages, pages, page_entries, unroll, flags, L, x, y, s);
}

extern "C" int edgpu_spmv_paged(const edgpu_csr* h, const void* pages, int64_t n_pages, int page_entries, int unroll,
                                int flags, const double* x, double* y, int R, void* stream) {
  return spmv_paged_impl<double>(h, pages, n_pages, page_entries, unroll, flags, x, y, R, (cudaStream_t)stream);
}

extern "C" int edgpu_spmv_paged_c64(const edgpu_csr* h, const void* pages, int64_t n_pages, int page_entries,
                                    int unroll, int flags, const float* x, float* y, int R, void* stream) {
  return spmv_paged_impl<float>(h, pages, n_pages, page_entries, unroll, flags, x, y, R, (cudaStream_t)stream);
}
