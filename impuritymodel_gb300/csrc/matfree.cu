// Matrix-free H·v on a sorted sector basis (edgpu_hv_diag, edgpu_hv_matfree[_c64]).
//
// y_i = sum_j H_ij x_j with H_ij = <b_i|H|b_j> = conj(<b_j|H|b_i>): row i is the conjugate of
// H applied to the single product state b_i, restricted to the sector (upstream builds the
// same numbers column by column with applyOp, impurityModel/ed/finite.py:1514-1693).  No
// matrix is stored:
//   * the diagonal d_i (all terms that map a state onto itself) is summed once per basis
//     state by edgpu_hv_diag, O(n) like a vector;
//   * every other term creates an electron in some orbital k that it does not annihilate, so
//     it can act on b_i only when orbital k is empty in b_i.  The off-diagonal terms come
//     bucketed by that key orbital; a warp serves one row, finds the empty orbitals of b_i
//     (a few of several hundred in these models) and applies only the terms of their buckets,
//     looks each result up in an open-addressing hash of the basis (edgpu_state_hash_build;
//     binary search of the sorted basis when no table is given) and collects (column, conj(h))
//     pairs in shared memory; then its lanes gather the x rows of the pairs, L lanes per pair
//     (16 bytes each), and the partial sums of the row groups are added with xor shuffles.
// The matrix-free product therefore costs term applications and L2 gathers, no CSR traffic.
#include "common.cuh"

namespace edgpu {
namespace {

template <typename T>
struct MfPack;
template <>
struct MfPack<float> {
  using type = float4;
  static constexpr int runs = 2;
};
template <>
struct MfPack<double> {
  using type = double2;
  static constexpr int runs = 1;
};

// Open-addressing hash of product states (edgpu_state_hash_build): slot -> basis index or -1,
// linear probing in a power-of-two table at most half full, so a lookup is one or two table
// reads and one basis read instead of ~log2(n) dependent basis reads of a binary search.
template <int W>
__device__ __forceinline__ uint64_t state_hash(const uint64_t (&s)[W]) {
  uint64_t h = 0x243F6A8885A308D3ull;
#pragma unroll
  for (int q = 0; q < W; ++q) {
    h ^= s[q] + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 31;
  }
  return h;
}

template <int W>
__global__ void state_hash_insert_kernel(const uint64_t* __restrict__ basis, int64_t n, int32_t* table,
                                         uint64_t mask) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t s[W];
  load_state<W>(basis + i * W, s);
  uint64_t slot = state_hash<W>(s) & mask;
  for (uint64_t probe = 0; probe <= mask; ++probe) {
    if (atomicCAS(reinterpret_cast<int*>(table + slot), -1, (int)i) == -1) return;
    slot = (slot + 1) & mask;
  }
}

template <int W>
__device__ __forceinline__ int64_t hash_find(const uint64_t* __restrict__ basis, const int32_t* __restrict__ table,
                                             uint64_t mask, const uint64_t (&key)[W]) {
  uint64_t slot = state_hash<W>(key) & mask;
  for (uint64_t probe = 0; probe <= mask; ++probe) {
    const int32_t idx = __ldg(table + slot);
    if (idx < 0) return -1;
    if (state_eq<W>(key, basis + (int64_t)idx * W)) return idx;
    slot = (slot + 1) & mask;
  }
  return -1;
}

constexpr int kMfWarps = 8;      // warps (rows in flight) per block
constexpr int kMfList = 256;     // (column, value) pairs buffered per warp

// d[i] = sum of the diagonal terms' contributions to <b_i|H|b_i> (sign from the term's
// transpositions), summed in term order.
template <int W>
__global__ void hv_diag_kernel(int64_t n, const uint64_t* __restrict__ basis, int n_terms,
                               const uint64_t* __restrict__ ops, const double2* __restrict__ coeff, double* d) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t s0[W];
  load_state<W>(basis + i * W, s0);
  double acc = 0.0;
  for (int t = 0; t < n_terms; ++t) {
    uint64_t s[W];
#pragma unroll
    for (int q = 0; q < W; ++q) s[q] = s0[q];
    int parity = 0;
    if (!apply_term<W>(s, __ldg(ops + t), parity)) continue;
    const double c = __ldg(&coeff[t].x);
    acc += (parity & 1) ? -c : c;
  }
  d[i] = acc;
}

template <int W, typename T, bool CPLX, int L>
__global__ void __launch_bounds__(32 * kMfWarps)
    hv_matfree_kernel(int64_t n, const uint64_t* __restrict__ basis, const int32_t* __restrict__ table,
                      uint64_t table_mask, int n_orb, const int32_t* __restrict__ bucket,
                      const uint64_t* __restrict__ ops, const double2* __restrict__ coeff, Restr restr,
                      const double* __restrict__ diag, double shift, const typename MfPack<T>::type* __restrict__ X,
                      typename MfPack<T>::type* __restrict__ Y) {
  using P = typename MfPack<T>::type;
  constexpr int RV = MfPack<T>::runs;
  constexpr int C = 32 / L;
  __shared__ int32_t lcol[kMfWarps][kMfList];
  __shared__ T lre[kMfWarps][kMfList];
  __shared__ T lim[kMfWarps][kMfList];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int grp = lane / L, sub = lane - grp * L;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nw) {
    uint64_t s0[W];
    load_state<W>(basis + i * W, s0);
    T ar[RV], ai[RV];
    {
      // diagonal: (d_i - shift) x_i, added by group 0 only
      const T dd = (T)(diag[i] - shift);
      const P xi = grp == 0 ? __ldg(X + i * L + sub) : P{};
      const T* xs = reinterpret_cast<const T*>(&xi);
#pragma unroll
      for (int q = 0; q < RV; ++q) {
        ar[q] = grp == 0 ? dd * xs[2 * q] : T(0);
        ai[q] = grp == 0 ? dd * xs[2 * q + 1] : T(0);
      }
    }
    int cnt = 0;  // pairs in the warp's list (warp-uniform)
    auto drain = [&]() {
      __syncwarp();
      for (int e0 = 0; e0 < cnt; e0 += C) {
        const int e = e0 + grp;
        if (e < cnt) {
          const P xv = __ldg(X + (int64_t)lcol[wib][e] * L + sub);
          const T hr = lre[wib][e], hi = lim[wib][e];
          const T* xs = reinterpret_cast<const T*>(&xv);
#pragma unroll
          for (int q = 0; q < RV; ++q) {
            const T xr = xs[2 * q], xq = xs[2 * q + 1];
            ar[q] += hr * xr;
            ai[q] += hr * xq;
            if (CPLX) {
              ar[q] -= hi * xq;
              ai[q] += hi * xr;
            }
          }
        }
      }
      __syncwarp();
      cnt = 0;
    };
    // empty orbitals of b_i, lowest first; each selects its bucket of off-diagonal terms
    for (int q = 0; q < W; ++q) {
      uint64_t empty = ~s0[q];
      const int base = 64 * q;
      if (base + 64 > n_orb) empty &= n_orb - base >= 64 ? ~0ull : (n_orb <= base ? 0ull : (~0ull << (64 - (n_orb - base))));
      while (empty) {
        const int bit = __clzll(empty);  // orbital base + bit (bit 63 - b holds orbital b)
        empty &= ~(1ull << (63 - bit));
        const int k = base + bit;
        const int t0 = __ldg(bucket + k), t1 = __ldg(bucket + k + 1);
        for (int tb = t0; tb < t1; tb += 32) {
          const int t = tb + lane;
          bool ok = false;
          int64_t j = -1;
          T vr = T(0), vi = T(0);
          if (t < t1) {
            uint64_t s[W];
#pragma unroll
            for (int w = 0; w < W; ++w) s[w] = s0[w];
            int parity = 0;
            if (apply_term<W>(s, __ldg(ops + t), parity) && restr_ok<W>(restr, s)) {
              j = table ? hash_find<W>(basis, table, table_mask, s) : find_state<W>(basis, n, s);
              if (j >= 0) {
                const double2 c = coeff[t];
                const double sg = (parity & 1) ? -1.0 : 1.0;
                vr = (T)(sg * c.x);
                vi = (T)(-sg * c.y);  // conj: row i of H is H|b_i> conjugated
                ok = true;
              }
            }
          }
          const unsigned m = __ballot_sync(0xffffffffu, ok);
          const int nv = __popc(m);
          if (cnt + nv > kMfList) drain();
          if (ok) {
            const int pos = cnt + __popc(m & ((1u << lane) - 1u));
            lcol[wib][pos] = (int32_t)j;
            lre[wib][pos] = vr;
            lim[wib][pos] = vi;
          }
          cnt += nv;
        }
      }
    }
    drain();
#pragma unroll
    for (int o = L; o < 32; o <<= 1)
#pragma unroll
      for (int q = 0; q < RV; ++q) {
        ar[q] += __shfl_xor_sync(0xffffffffu, ar[q], o);
        ai[q] += __shfl_xor_sync(0xffffffffu, ai[q], o);
      }
    if (grp == 0) {
      P out;
      T* os = reinterpret_cast<T*>(&out);
#pragma unroll
      for (int q = 0; q < RV; ++q) {
        os[2 * q] = ar[q];
        os[2 * q + 1] = ai[q];
      }
      Y[i * L + sub] = out;
    }
  }
}

template <int W, typename T, bool CPLX>
int launch_matfree_l(int L, int64_t n, const uint64_t* basis, const int32_t* table, uint64_t table_mask, int n_orb,
                     const int32_t* bucket, const uint64_t* ops,
                     const double2* coeff, const Restr& r, const double* diag, double shift, const void* x, void* y,
                     cudaStream_t s) {
  using P = typename MfPack<T>::type;
  int64_t blocks = (n + kMfWarps - 1) / kMfWarps;
  const int64_t cap = (int64_t)grid_cap() * 16;
  if (blocks > cap) blocks = cap;
  const P* X = reinterpret_cast<const P*>(x);
  P* Y = reinterpret_cast<P*>(y);
#define EDGPU_MF_CASE(LL)                                                                                  \
  case LL:                                                                                                 \
    hv_matfree_kernel<W, T, CPLX, LL><<<(unsigned)blocks, 32 * kMfWarps, 0, s>>>(n, basis, table, table_mask, \
                                                                                 n_orb, bucket,            \
                                                                                 ops, coeff, r, diag,      \
                                                                                 shift, X, Y);             \
    break;
  switch (L) {
    EDGPU_MF_CASE(1)
    EDGPU_MF_CASE(2)
    EDGPU_MF_CASE(4)
    EDGPU_MF_CASE(8)
    EDGPU_MF_CASE(16)
    EDGPU_MF_CASE(32)
    default:
      return EDGPU_ERR_ARG;
  }
#undef EDGPU_MF_CASE
  note_launch();
  return check_launch();
}

template <typename T>
int hv_matfree_impl(int n_words, const uint64_t* basis, int64_t n, const int32_t* table, int64_t table_size,
                    int n_orb, const int32_t* bucket,
                    const edgpu_terms* terms, int complex_terms, const edgpu_restrictions* restr, const double* diag,
                    double shift, const void* x, void* y, int R, cudaStream_t s) {
  if (!basis || n < 1 || !bucket || !terms || !diag || !x || !y || R < 1) return EDGPU_ERR_ARG;
  if (n_orb < 1 || n_orb > 64 * n_words || n_words < 1 || n_words > EDGPU_MAX_WORDS) return EDGPU_ERR_ARG;
  if (table && (table_size < 2 * n || (table_size & (table_size - 1)))) return EDGPU_ERR_ARG;
  const uint64_t mask = table ? (uint64_t)table_size - 1 : 0;
  if (terms->n_terms > 0 && (!terms->ops || !terms->coeff)) return EDGPU_ERR_ARG;
  constexpr int RV = MfPack<T>::runs;
  if (R % RV) return EDGPU_ERR_ARG;
  const int L = R / RV;
  if (L > 32 || (32 % L)) return EDGPU_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15) return EDGPU_ERR_ARG;
  const Restr r = make_restr(restr);
  const double2* coeff = reinterpret_cast<const double2*>(terms->coeff);
  EDGPU_DISPATCH_W(n_words, return complex_terms
                                ? launch_matfree_l<W, T, true>(L, n, basis, table, mask, n_orb, bucket, terms->ops,
                                                               coeff, r, diag, shift, x, y, s)
                                : launch_matfree_l<W, T, false>(L, n, basis, table, mask, n_orb, bucket, terms->ops,
                                                                coeff, r, diag, shift, x, y, s));
  return EDGPU_ERR_ARG;
}

}  // namespace
}  // namespace edgpu

using namespace edgpu;

extern "C" int edgpu_hv_diag(int n_words, const uint64_t* basis, int64_t n, const edgpu_terms* diag_terms,
                             double* d, void* stream) {
  if (!basis || n < 1 || !diag_terms || !d) return EDGPU_ERR_ARG;
  if (diag_terms->n_terms > 0 && (!diag_terms->ops || !diag_terms->coeff)) return EDGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  const double2* coeff = reinterpret_cast<const double2*>(diag_terms->coeff);
  EDGPU_DISPATCH_W(n_words, hv_diag_kernel<W><<<blocks, 256, 0, s>>>(n, basis, diag_terms->n_terms, diag_terms->ops,
                                                                     coeff, d));
  note_launch();
  return check_launch();
}

extern "C" int edgpu_state_hash_build(int n_words, const uint64_t* basis, int64_t n, int32_t* table,
                                      int64_t table_size, void* stream) {
  if (!basis || !table || n < 1 || n >= (1ll << 31) || table_size < 2 * n || (table_size & (table_size - 1)))
    return EDGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(table, 0xFF, sizeof(int32_t) * (size_t)table_size, s) != cudaSuccess) return EDGPU_ERR_CUDA;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  EDGPU_DISPATCH_W(n_words, state_hash_insert_kernel<W><<<blocks, 256, 0, s>>>(basis, n, table,
                                                                               (uint64_t)table_size - 1));
  note_launch();
  return check_launch();
}

extern "C" int edgpu_hv_matfree(int n_words, const uint64_t* basis, int64_t n, const int32_t* table,
                                int64_t table_size, int n_orb, const int32_t* bucket,
                                const edgpu_terms* offdiag_terms, int complex_terms,
                                const edgpu_restrictions* restr, const double* diag, double shift, const double* x,
                                double* y, int R, void* stream) {
  return hv_matfree_impl<double>(n_words, basis, n, table, table_size, n_orb, bucket, offdiag_terms, complex_terms,
                                 restr, diag, shift, x, y, R, (cudaStream_t)stream);
}

extern "C" int edgpu_hv_matfree_c64(int n_words, const uint64_t* basis, int64_t n, const int32_t* table,
                                    int64_t table_size, int n_orb, const int32_t* bucket,
                                    const edgpu_terms* offdiag_terms, int complex_terms,
                                    const edgpu_restrictions* restr, const double* diag, double shift,
                                    const float* x, float* y, int R, void* stream) {
  return hv_matfree_impl<float>(n_words, basis, n, table, table_size, n_orb, bucket, offdiag_terms, complex_terms,
                                restr, diag, shift, x, y, R, (cudaStream_t)stream);
}
