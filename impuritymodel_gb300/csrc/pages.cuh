// Entries of the paged H·v layout (edgpu_spmv_pages_build): column index and value of one
// CSR entry, or a slice header (column -2 - row, or INT_MIN for none) whose flag marks a
// heavy row, or padding (column -1).  Shared by the paged kernels of spmv.cu and spmv_tma.cu.
#pragma once
#include <cstdint>

namespace edgpu {

template <typename T, bool VALC>
struct Ent;
template <>
struct __align__(8) Ent<float, false> {
  int32_t c;
  float v;
  __device__ __forceinline__ int flag() const { return __float_as_int(v); }
  __device__ __forceinline__ void set_flag(int f) { v = __int_as_float(f); }
};
template <>
struct __align__(16) Ent<double, false> {
  int32_t c;
  int32_t aux;
  double v;
  __device__ __forceinline__ int flag() const { return aux; }
  __device__ __forceinline__ void set_flag(int f) { aux = f; }
};
template <>
struct __align__(16) Ent<float, true> {
  int32_t c;
  int32_t aux;
  float vr, vi;
  __device__ __forceinline__ int flag() const { return aux; }
  __device__ __forceinline__ void set_flag(int f) { aux = f; }
};

}  // namespace edgpu
