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
    for (int o = NW / 2; o > 0; o >>= 1)
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
