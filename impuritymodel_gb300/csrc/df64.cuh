// Double-float arithmetic shared by the double-float kernels.
#pragma once

#include <cuda_runtime.h>

namespace edgpu {

// ---------------------------------------------------------------------------------------
// Double-float ("df64") arithmetic: a value is an unevaluated sum hi + lo of two floats,
// about 48 significand bits.  Error-free transformations (Knuth's two-sum, Dekker's
// fast two-sum, the FMA two-product) use __fadd_rn/__fsub_rn/__fmul_rn, which the compiler
// never contracts into FMAs, so the transformations stay exact.  On GB300 a df64
// multiply-add costs ~12 FP32 instructions against one FP64 FMA issued at 1/64 of the FP32
// rate, so it is several times faster than FP64 for the Krylov recurrences.
// ---------------------------------------------------------------------------------------
struct dfl {
  float hi, lo;
};

__device__ __forceinline__ dfl df_split(double a) {
  const float hi = (float)a;
  return {hi, (float)(a - (double)hi)};
}

__device__ __forceinline__ double df_val(dfl a) { return (double)a.hi + (double)a.lo; }

// |a| >= |b| or a == 0
__device__ __forceinline__ dfl df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dfl df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

// acc + a * b
__device__ __forceinline__ dfl df_fma(dfl acc, dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float pe = fmaf(a.hi, b.hi, -p);
  pe = fmaf(a.hi, b.lo, pe);
  pe = fmaf(a.lo, b.hi, pe);
  const dfl s = df_two_sum(acc.hi, p);
  return df_fast_two_sum(s.hi, __fadd_rn(__fadd_rn(s.lo, pe), acc.lo));
}

__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}

__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
  const dfl s = df_two_sum(a.hi, b.hi);
  return df_fast_two_sum(s.hi, __fadd_rn(__fadd_rn(s.lo, a.lo), b.lo));
}

// Deterministic double-float block sum on the FP32 pipe (fixed shuffle tree, then warp 0
// over the NW per-warp partials), broadcast to every thread, with two barriers: consecutive sums must
// alternate between two partial buffers of 33 entries, so that a sum never overwrites the
// partials that a slower thread may still be reading from the previous one (every thread
// reads the previous result before it reaches the next sum's first barrier).
constexpr int kDfRed = 80;  // two 40-entry partial buffers
// first shuffle distance of a tree over NW partials: half the next power of two, so that a
// warp count that is not a power of two (5 or 6 warps) still adds every partial
__host__ __device__ constexpr int df_tree_top(int nw) {
  int p = 1;
  while (p < nw) p <<= 1;
  return p / 2;
}
template <int NW>
__device__ __forceinline__ dfl df_block_sum2(dfl v, dfl* buf) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v = df_add(v, {__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)});
  if (lane == 0) buf[warp] = v;
  __syncthreads();
  if (warp == 0) {
    dfl t = lane < NW ? buf[lane] : dfl{0.f, 0.f};
#pragma unroll
    for (int o = df_tree_top(NW); o > 0; o >>= 1)
      t = df_add(t, {__shfl_down_sync(0xffffffffu, t.hi, o), __shfl_down_sync(0xffffffffu, t.lo, o)});
    if (lane == 0) buf[32] = t;
  }
  __syncthreads();
  return buf[32];
}

// Double-float running sum s + c with the compensation c left unnormalised until the end:
// two-sum keeps the high parts exact, and the FP32 sum of the (small) low parts costs a
// relative 2^-48 per term like a full double-float add, for 12 instructions per multiply-add
// instead of 15.
struct dacc {
  float s, c;
};

// a += h * (xh + xl)
__device__ __forceinline__ void dacc_fma(dacc& a, dfl h, float xh, float xl) {
  const float p = __fmul_rn(h.hi, xh);
  float pe = fmaf(h.hi, xh, -p);
  pe = fmaf(h.hi, xl, pe);
  pe = fmaf(h.lo, xh, pe);
  const dfl t = df_two_sum(a.s, p);
  a.s = t.hi;
  a.c = __fadd_rn(a.c, __fadd_rn(t.lo, pe));
}

__device__ __forceinline__ dfl dacc_val(dacc a) { return df_two_sum(a.s, a.c); }

// sqrt(a) for a > 0: FP32 square root s, then one Newton correction (a - s^2) / (2 s) with
// s^2 formed exactly by the FMA two-product (Dekker's double-length square root).
__device__ __forceinline__ dfl df_sqrt(dfl a) {
  if (!(a.hi > 0.f)) return {a.hi == 0.f ? 0.f : __fsqrt_rn(a.hi), 0.f};
  const float s = __fsqrt_rn(a.hi);
  const float p = __fmul_rn(s, s);
  const float pe = fmaf(s, s, -p);
  const float r = __fdiv_rn(__fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), a.lo), __fadd_rn(s, s));
  return df_fast_two_sum(s, r);
}

// 1 / b for b != 0: FP32 reciprocal r, then one Newton step r + r (1 - b r) with the
// residual 1 - b r formed from the exact product b.hi * r.
__device__ __forceinline__ dfl df_rcp(dfl b) {
  const float r = __fdiv_rn(1.f, b.hi);
  const float p = __fmul_rn(b.hi, r);
  const float pe = fmaf(b.hi, r, -p);
  const float e = __fsub_rn(__fsub_rn(__fsub_rn(1.f, p), pe), __fmul_rn(b.lo, r));
  return df_fast_two_sum(r, __fmul_rn(r, e));
}

}  // namespace edgpu

namespace edgpu {

// ---------------------------------------------------------------------------------------
// Two independent double-floats (the real and imaginary parts of a complex number) in packed
// float2 registers.  GB300's packed FP32 instructions (__fadd2_rn / __fmul2_rn / __ffma2_rn,
// per component the same as __fadd_rn / __fmul_rn / __fmaf_rn) carry both in one issue, so
// each operation below is its scalar counterpart, component by component, at half the
// instruction count.
// ---------------------------------------------------------------------------------------
struct dfl2 {
  float2 hi, lo;
};

__device__ __forceinline__ float2 f2neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 f2dup(float a) { return make_float2(a, a); }

__device__ __forceinline__ dfl2 df2_fast_two_sum(float2 a, float2 b) {
  const float2 s = __fadd2_rn(a, b);
  return {s, __fadd2_rn(b, f2neg(__fadd2_rn(s, f2neg(a))))};
}

__device__ __forceinline__ dfl2 df2_two_sum(float2 a, float2 b) {
  const float2 s = __fadd2_rn(a, b);
  const float2 bb = __fadd2_rn(s, f2neg(a));
  return {s, __fadd2_rn(__fadd2_rn(a, f2neg(__fadd2_rn(s, f2neg(bb)))), __fadd2_rn(b, f2neg(bb)))};
}

// acc + a * b, b the same double-float for both components
__device__ __forceinline__ dfl2 df2_fma_s(dfl2 acc, dfl2 a, dfl b) {
  const float2 bh = f2dup(b.hi), bl = f2dup(b.lo);
  const float2 p = __fmul2_rn(a.hi, bh);
  float2 pe = __ffma2_rn(a.hi, bh, f2neg(p));
  pe = __ffma2_rn(a.hi, bl, pe);
  pe = __ffma2_rn(a.lo, bh, pe);
  const dfl2 s = df2_two_sum(acc.hi, p);
  return df2_fast_two_sum(s.hi, __fadd2_rn(__fadd2_rn(s.lo, pe), acc.lo));
}

__device__ __forceinline__ dfl2 df2_mul_s(dfl2 a, dfl b) {
  const float2 bh = f2dup(b.hi), bl = f2dup(b.lo);
  const float2 p = __fmul2_rn(a.hi, bh);
  float2 e = __ffma2_rn(a.hi, bh, f2neg(p));
  e = __ffma2_rn(a.hi, bl, e);
  e = __ffma2_rn(a.lo, bh, e);
  return df2_fast_two_sum(p, e);
}

// Packed running sums (s + c per component, as dacc)
struct dacc2 {
  float2 s, c;
};

// a += h * x, h the same double-float for both components, x = (xh + xl) per component
__device__ __forceinline__ void dacc2_fma(dacc2& a, dfl h, float2 xh, float2 xl) {
  const float2 hh = f2dup(h.hi), hl = f2dup(h.lo);
  const float2 p = __fmul2_rn(hh, xh);
  float2 pe = __ffma2_rn(hh, xh, f2neg(p));
  pe = __ffma2_rn(hh, xl, pe);
  pe = __ffma2_rn(hl, xh, pe);
  const dfl2 t = df2_two_sum(a.s, p);
  a.s = t.hi;
  a.c = __fadd2_rn(a.c, __fadd2_rn(t.lo, pe));
}

// a += h * x componentwise (h a pair)
__device__ __forceinline__ void dacc2_fma2(dacc2& a, dfl2 h, float2 xh, float2 xl) {
  const float2 p = __fmul2_rn(h.hi, xh);
  float2 pe = __ffma2_rn(h.hi, xh, f2neg(p));
  pe = __ffma2_rn(h.hi, xl, pe);
  pe = __ffma2_rn(h.lo, xh, pe);
  const dfl2 t = df2_two_sum(a.s, p);
  a.s = t.hi;
  a.c = __fadd2_rn(a.c, __fadd2_rn(t.lo, pe));
}

__device__ __forceinline__ dfl2 dacc2_val(dacc2 a) { return df2_two_sum(a.s, a.c); }

// sum of the two components of a packed running sum, as one double-float
__device__ __forceinline__ dfl dacc2_total(dacc2 a) {
  const dfl2 v = dacc2_val(a);
  return df_add({v.hi.x, v.lo.x}, {v.hi.y, v.lo.y});
}

}  // namespace edgpu
