// Shared device helpers of the edgpu engine: packed product states, fermionic signs,
// restriction checks, lexicographic comparison and binary search over sorted bases.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/edgpu.h"

namespace edgpu {

constexpr int kWarp = 32;

// Dispatch a runtime word count (1..8) to a template instantiation.
#define EDGPU_DISPATCH_W(nw, ...)                       \
  switch (nw) {                                         \
    case 1: { constexpr int W = 1; __VA_ARGS__; break; } \
    case 2: { constexpr int W = 2; __VA_ARGS__; break; } \
    case 3: { constexpr int W = 3; __VA_ARGS__; break; } \
    case 4: { constexpr int W = 4; __VA_ARGS__; break; } \
    case 5: { constexpr int W = 5; __VA_ARGS__; break; } \
    case 6: { constexpr int W = 6; __VA_ARGS__; break; } \
    case 7: { constexpr int W = 7; __VA_ARGS__; break; } \
    case 8: { constexpr int W = 8; __VA_ARGS__; break; } \
    default: return EDGPU_ERR_ARG;                      \
  }

inline int grid_cap() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 148;
  }
  return sms;
}

// Running count of kernels this library launched (edgpu_launch_count).
void note_launch();

inline int check_launch() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? EDGPU_OK : EDGPU_ERR_CUDA;
}

// Restriction set passed by value into kernels.
struct Restr {
  int n;
  int lo[EDGPU_MAX_RESTRICTIONS];
  int hi[EDGPU_MAX_RESTRICTIONS];
  uint64_t mask[EDGPU_MAX_RESTRICTIONS][EDGPU_MAX_WORDS];
};

inline Restr make_restr(const edgpu_restrictions* r) {
  Restr o{};
  o.n = 0;
  if (r) {
    o.n = r->n;
    for (int k = 0; k < r->n && k < EDGPU_MAX_RESTRICTIONS; ++k) {
      o.lo[k] = r->lo[k];
      o.hi[k] = r->hi[k];
      for (int q = 0; q < EDGPU_MAX_WORDS; ++q) o.mask[k][q] = r->mask[k][q];
    }
  }
  return o;
}

template <int W>
__device__ __forceinline__ bool restr_ok(const Restr& r, const uint64_t (&s)[W]) {
  for (int k = 0; k < r.n; ++k) {
    int c = 0;
#pragma unroll
    for (int q = 0; q < W; ++q) c += __popcll(s[q] & r.mask[k][q]);
    if (c < r.lo[k] || c > r.hi[k]) return false;
  }
  return true;
}

template <int W>
__device__ __forceinline__ void load_state(const uint64_t* p, uint64_t (&s)[W]) {
#pragma unroll
  for (int q = 0; q < W; ++q) s[q] = p[q];
}

template <int W>
__device__ __forceinline__ void store_state(uint64_t* p, const uint64_t (&s)[W]) {
#pragma unroll
  for (int q = 0; q < W; ++q) p[q] = s[q];
}

template <int W>
__device__ __forceinline__ bool state_eq(const uint64_t (&a)[W], const uint64_t* b) {
  bool eq = true;
#pragma unroll
  for (int q = 0; q < W; ++q) eq &= (a[q] == b[q]);
  return eq;
}

// -1 / 0 / +1 lexicographic comparison of a (registers) with b (memory).
template <int W>
__device__ __forceinline__ int state_cmp(const uint64_t (&a)[W], const uint64_t* b) {
#pragma unroll
  for (int q = 0; q < W; ++q) {
    uint64_t bq = b[q];
    if (a[q] != bq) return a[q] < bq ? -1 : 1;
  }
  return 0;
}

template <int W>
__device__ __forceinline__ int state_cmp_mm(const uint64_t* a, const uint64_t* b) {
#pragma unroll
  for (int q = 0; q < W; ++q) {
    uint64_t aq = a[q], bq = b[q];
    if (aq != bq) return aq < bq ? -1 : 1;
  }
  return 0;
}

// First index i in sorted basis[0..n) with basis[i] >= key.
template <int W>
__device__ __forceinline__ int64_t lower_bound_state(const uint64_t* basis, int64_t n, const uint64_t (&key)[W]) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (state_cmp<W>(key, basis + mid * W) > 0)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

template <int W>
__device__ __forceinline__ int64_t find_state(const uint64_t* basis, int64_t n, const uint64_t (&key)[W]) {
  int64_t p = lower_bound_state<W>(basis, n, key);
  if (p < n && state_cmp<W>(key, basis + p * W) == 0) return p;
  return -1;
}

// Apply one packed term (up to 4 elementary operators, right to left) to state s.
// Returns false if Pauli-blocked; otherwise s holds the new state and parity the number
// of transpositions (sign = (-1)^parity).  Sign rule of upstream create/remove.ubitarray:
// (-1)^(number of occupied orbitals with smaller index), evaluated before the bit flip.
template <int W>
__device__ __forceinline__ bool apply_term(uint64_t (&s)[W], uint64_t ops, int& parity) {
#pragma unroll
  for (int k = 3; k >= 0; --k) {
    const uint32_t op = (uint32_t)(ops >> (16 * k)) & 0xFFFFu;
    if (!(op & 0x8000u)) continue;
    const int orb = (int)(op & 0x3FFu);
    const bool cre = (op & 0x4000u) != 0;
    const int wi = orb >> 6;
    const int bi = orb & 63;
    const uint64_t m = 1ull << (63 - bi);
    const uint64_t above = bi ? (~0ull << (64 - bi)) : 0ull;
    uint64_t word = 0;
    int cnt = 0;
#pragma unroll
    for (int q = 0; q < W; ++q) {
      if (q == wi) word = s[q];
      if (q < wi) cnt += __popcll(s[q]);
    }
    const bool occ = (word & m) != 0;
    if (occ == cre) return false;
    cnt += __popcll(word & above);
    parity += cnt;
#pragma unroll
    for (int q = 0; q < W; ++q)
      if (q == wi) s[q] ^= m;
  }
  return true;
}

// |v|^2 as CPython computes abs(v)**2: hypot first, then square.
__device__ __forceinline__ double abs2_py(double re, double im) {
  double a = hypot(re, im);
  return __dmul_rn(a, a);
}

}  // namespace edgpu
