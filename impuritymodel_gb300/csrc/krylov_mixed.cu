// Batched reorthogonalised Lanczos pieces for large sectors, vectors in complex64 or
// complex128 with FP64-accumulated reductions (edgpu_krylov_dot, edgpu_krylov_project,
// edgpu_krylov_normalize).
//
// R runs share each call; a Krylov vector is [n][R] (run fastest), the basis V[m][n][R].
// Step j of a run set, with w = H v_j from any H·v kernel:
//   h  = V[0..j]^H w,  w -= V h          (pass 1: alpha_j = Re h_j, the three-term update and
//   h' = V[0..j]^H w,  w -= V h'          the reorthogonalisation in one classical Gram-Schmidt)
//   beta_j = |w|,  v_{j+1} = w / beta_j   (pass 2 ensures orthogonality to working precision)
// This replaces upstream's unreorthogonalised recurrence (impurityModel/ed/finite.py:1897-1995)
// for sectors of 1e5..1e6 states, where a complex64 recurrence without reorthogonalisation
// loses orthogonality within a few dozen steps.
//
// Every pass streams V once from HBM, so the kernels are built for bandwidth: each thread
// moves 16 bytes per access (two complex64 runs, or one complex128); the dot streams its
// lanes through a cp.async ring in shared memory (several row steps in flight per thread
// without holding them in registers), and the projection loads V with the streaming
// (evict-first) policy, unrolled over vectors so that several 16-byte loads are in flight.
//
// Reductions: each thread sums its products over up to 8 rows in the vector type, then adds
// that partial into an FP64 accumulator; blocks reduce in shared memory in a fixed tree and a
// second launch adds the per-block partials in a fixed order (deterministic, FP64 throughout
// above the first eight products).  Projections and scalings run in the vector type with the
// FP64 coefficients rounded to it.
#include <algorithm>

#include "common.cuh"

namespace edgpu {
namespace {

constexpr int kKmThreads = 256;
constexpr int kKmChunk = 8;  // products summed in the vector type before an FP64 add
constexpr int KD = 4;        // Krylov vectors per dot block (w is read once for all of them)
constexpr int KB = 2048;     // projection coefficients staged in shared memory per round

// One thread's lane: VW complex numbers of one row (consecutive runs).
template <typename T, int VW>
struct Lane;
template <>
struct Lane<float, 2> {
  using type = float4;
};
template <>
struct Lane<float, 1> {
  using type = float2;
};
template <>
struct Lane<double, 1> {
  using type = double2;
};

__device__ __forceinline__ void unpack(const float4& u, float (&re)[2], float (&im)[2]) {
  re[0] = u.x;
  im[0] = u.y;
  re[1] = u.z;
  im[1] = u.w;
}
__device__ __forceinline__ void unpack(const float2& u, float (&re)[1], float (&im)[1]) {
  re[0] = u.x;
  im[0] = u.y;
}
__device__ __forceinline__ void unpack(const double2& u, double (&re)[1], double (&im)[1]) {
  re[0] = u.x;
  im[0] = u.y;
}
__device__ __forceinline__ float4 pack(const float (&re)[2], const float (&im)[2]) {
  return make_float4(re[0], im[0], re[1], im[1]);
}
__device__ __forceinline__ float2 pack(const float (&re)[1], const float (&im)[1]) {
  return make_float2(re[0], im[0]);
}
__device__ __forceinline__ double2 pack(const double (&re)[1], const double (&im)[1]) {
  return make_double2(re[0], im[0]);
}

__device__ __forceinline__ void add_to(double& a, const double& b) { a += b; }
__device__ __forceinline__ void add_to(double2& a, const double2& b) {
  a.x += b.x;
  a.y += b.y;
}

// Fixed-order tree over the index rr of the values red[rr * width + c], rr < rows; every
// thread of the block calls it (it synchronises).
template <typename A>
__device__ __forceinline__ void tree_rows(A* red, int tid, int rr, int rows, int width) {
  for (int h = (rows + 1) / 2, len = rows; len > 1; len = h, h = (h + 1) / 2) {
    if (rr + h < len) add_to(red[tid], red[tid + h * width]);
    __syncthreads();
  }
}

// Asynchronous 16- or 8-byte copies global -> shared (the thread's own lane of a stage), with
// an L2 eviction-priority policy: the basis vectors stream through once (evict first), w is
// read again by every vector group of the pass (evict last).
template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem, uint64_t pol) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;\n" ::"r"(d), "l"(gmem), "l"(pol)
                 : "memory");
  else
    asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 8, %2;\n" ::"r"(d), "l"(gmem), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ uint64_t l2_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;\n" : "=l"(p));
  return p;
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

constexpr int kDotStages = 3;  // row steps of (w, KD vectors) in flight per thread

// Shared memory of the dot kernel: [stage][KD + 1][thread] lanes.
template <typename T, int VW>
constexpr size_t dot_smem_bytes() {
  return sizeof(typename Lane<T, VW>::type) * (size_t)kDotStages * (KD + 1) * kKmThreads;
}

// partial[k][b][r] = sum over block b's rows of conj(V[k][i][r]) * w[i][r], for the KD
// vectors k = blockIdx.y * KD + kk.  Lanes: tpr = R / VW threads per row.  Each thread
// streams its own lanes of w and of the KD vectors through a kDotStages-deep cp.async ring
// in shared memory (a thread reads back only what it copied itself, so no block barrier is
// needed inside the loop), which keeps kDotStages row steps of loads in flight per thread
// without holding them in registers.
template <typename T, int VW>
__global__ void __launch_bounds__(kKmThreads)
    krylov_dot_kernel(const typename Lane<T, VW>::type* __restrict__ V, int64_t stride_l, int m, int64_t n, int R,
                      const typename Lane<T, VW>::type* __restrict__ w, double2* __restrict__ partial) {
  using LT = typename Lane<T, VW>::type;
  extern __shared__ __align__(16) unsigned char km_smem[];
  LT* ring = reinterpret_cast<LT*>(km_smem);  // [kDotStages][KD + 1][kKmThreads]
  __shared__ double2 red[kKmThreads];
  const int tpr = R / VW, rpb = kKmThreads / tpr;
  const int tid = threadIdx.x;
  const int c = tid % tpr, rr = tid / tpr;
  const int k0 = blockIdx.y * KD;
  const int kn = m - k0 < KD ? m - k0 : KD;
  double sr[KD][VW], si[KD][VW];
#pragma unroll
  for (int kk = 0; kk < KD; ++kk)
#pragma unroll
    for (int v = 0; v < VW; ++v) sr[kk][v] = si[kk][v] = 0.0;
  const int64_t step = (int64_t)gridDim.x * rpb;
  const int64_t i0 = (int64_t)blockIdx.x * rpb + rr;
  const int64_t ns = (rr < rpb && i0 < n) ? (n - i0 + step - 1) / step : 0;  // this thread's row steps
  const uint64_t pol_v = l2_evict_first(), pol_w = l2_evict_last();
  auto issue = [&](int64_t s) {
    if (s < ns) {
      const int64_t e = (i0 + s * step) * tpr + c;
      LT* slot = ring + (size_t)(s % kDotStages) * (KD + 1) * kKmThreads + tid;
      cp_async<sizeof(LT)>(slot, w + e, pol_w);
#pragma unroll
      for (int kk = 0; kk < KD; ++kk)
        if (kk < kn)
          cp_async<sizeof(LT)>(slot + (kk + 1) * kKmThreads, V + (int64_t)(k0 + kk) * stride_l + e, pol_v);
    }
    cp_async_commit();  // one group per step, empty past the end, so the wait count holds
  };
#pragma unroll
  for (int s = 0; s < kDotStages - 1; ++s) issue(s);
  for (int64_t s0 = 0; s0 < ns; s0 += kKmChunk) {
    T cr[KD][VW], ci[KD][VW];
#pragma unroll
    for (int kk = 0; kk < KD; ++kk)
#pragma unroll
      for (int v = 0; v < VW; ++v) cr[kk][v] = ci[kk][v] = T(0);
    const int64_t s1 = s0 + kKmChunk < ns ? s0 + kKmChunk : ns;
    for (int64_t s = s0; s < s1; ++s) {
      issue(s + kDotStages - 1);
      cp_async_wait<kDotStages - 1>();  // step s has landed
      const LT* slot = ring + (size_t)(s % kDotStages) * (KD + 1) * kKmThreads + tid;
      T br[VW], bi[VW];
      unpack(slot[0], br, bi);
#pragma unroll
      for (int kk = 0; kk < KD; ++kk) {
        if (kk < kn) {
          T ar[VW], ai[VW];
          unpack(slot[(kk + 1) * kKmThreads], ar, ai);
#pragma unroll
          for (int v = 0; v < VW; ++v) {
            cr[kk][v] += ar[v] * br[v] + ai[v] * bi[v];
            ci[kk][v] += ar[v] * bi[v] - ai[v] * br[v];
          }
        }
      }
    }
#pragma unroll
    for (int kk = 0; kk < KD; ++kk)
#pragma unroll
      for (int v = 0; v < VW; ++v) {
        sr[kk][v] += (double)cr[kk][v];
        si[kk][v] += (double)ci[kk][v];
      }
  }
  cp_async_wait<0>();
#pragma unroll
  for (int kk = 0; kk < KD; ++kk) {
    if (kk < kn) {  // kn is the same for the whole block
#pragma unroll
      for (int v = 0; v < VW; ++v) {
        red[tid] = make_double2(sr[kk][v], si[kk][v]);
        __syncthreads();
        tree_rows(red, tid, rr, rpb, tpr);
        if (rr == 0) partial[((int64_t)(k0 + kk) * gridDim.x + blockIdx.x) * R + c * VW + v] = red[c];
        __syncthreads();
      }
    }
  }
}

// h[k][r] = sum over blocks b of partial[k][b][r]: one block per k; the blocks are split
// into kKmThreads / R interleaved slices summed in order, the slices added in a fixed tree.
__global__ void __launch_bounds__(kKmThreads) krylov_dot_reduce_kernel(const double2* __restrict__ partial, int nb,
                                                                      int R, double2* __restrict__ h) {
  __shared__ double2 red[kKmThreads];
  const int k = blockIdx.x, tid = threadIdx.x;
  const int r = tid % R, s = tid / R, S = kKmThreads / R;
  double2 acc = make_double2(0.0, 0.0);
  if (s < S)
    for (int b = s; b < nb; b += S) add_to(acc, partial[((int64_t)k * nb + b) * R + r]);
  red[tid] = acc;
  __syncthreads();
  tree_rows(red, tid, s, S, R);
  if (s == 0) h[(int64_t)k * R + r] = red[r];
}

// w[i][r] -= sum_k h[k][r] V[k][i][r]; with norms: per-block FP64 partials of |w[.][r]|^2
template <typename T, int VW>
__global__ void __launch_bounds__(kKmThreads)
    krylov_project_kernel(const typename Lane<T, VW>::type* __restrict__ V, int64_t stride_l, int m, int64_t n, int R,
                          const double2* __restrict__ h, typename Lane<T, VW>::type* __restrict__ w,
                          double* __restrict__ npart) {
  __shared__ T hre[KB], him[KB];
  __shared__ double red[kKmThreads];
  const int tpr = R / VW, rpb = kKmThreads / tpr;
  const int tid = threadIdx.x;
  const int c = tid % tpr, rr = tid / tpr;
  const int kpr = KB / R;  // vectors per staging round
  double nacc[VW];
#pragma unroll
  for (int v = 0; v < VW; ++v) nacc[v] = 0.0;
  const int64_t step = (int64_t)gridDim.x * rpb;
  for (int k0 = 0; k0 < m; k0 += kpr) {
    const int kc = (m - k0) < kpr ? (m - k0) : kpr;
    __syncthreads();
    for (int t = tid; t < kc * R; t += kKmThreads) {
      const double2 cf = h[(int64_t)k0 * R + t];
      hre[t] = (T)cf.x;
      him[t] = (T)cf.y;
    }
    __syncthreads();
    if (rr < rpb) {
      for (int64_t i = (int64_t)blockIdx.x * rpb + rr; i < n; i += step) {
        T wr[VW], wi[VW];
        unpack(w[i * tpr + c], wr, wi);
        const typename Lane<T, VW>::type* vp = V + (int64_t)k0 * stride_l + i * tpr + c;
#pragma unroll 8
        for (int k = 0; k < kc; ++k) {
          T vr[VW], vi[VW];
          unpack(__ldcs(vp + (int64_t)k * stride_l), vr, vi);
#pragma unroll
          for (int v = 0; v < VW; ++v) {
            const T hr = hre[k * R + c * VW + v], hi = him[k * R + c * VW + v];
            wr[v] -= hr * vr[v] - hi * vi[v];
            wi[v] -= hr * vi[v] + hi * vr[v];
          }
        }
        w[i * tpr + c] = pack(wr, wi);
        if (npart && k0 + kc >= m) {
#pragma unroll
          for (int v = 0; v < VW; ++v) nacc[v] += (double)wr[v] * wr[v] + (double)wi[v] * wi[v];
        }
      }
    }
  }
  if (!npart) return;  // the same for every thread of the launch
#pragma unroll
  for (int v = 0; v < VW; ++v) {
    red[tid] = nacc[v];
    __syncthreads();
    tree_rows(red, tid, rr, rpb, tpr);
    if (rr == 0) npart[(int64_t)blockIdx.x * R + c * VW + v] = red[c];
    __syncthreads();
  }
}

// beta[r] = sqrt(sum_b npart[b][r]) in a fixed order (one block); beta == 0 sets the status
__global__ void __launch_bounds__(kKmThreads) krylov_norm_reduce_kernel(const double* __restrict__ npart, int nb,
                                                                       int R, double* __restrict__ beta,
                                                                       int32_t* status) {
  __shared__ double red[kKmThreads];
  const int tid = threadIdx.x;
  const int r = tid % R, s = tid / R, S = kKmThreads / R;
  double acc = 0.0;
  if (s < S)
    for (int b = s; b < nb; b += S) acc += npart[(int64_t)b * R + r];
  red[tid] = acc;
  __syncthreads();
  tree_rows(red, tid, s, S, R);
  if (s == 0) {
    const double b = sqrt(red[r]);
    beta[r] = b;
    if (!(b > 0.0) && status) atomicExch(status, (int32_t)EDGPU_ERR_BREAKDOWN);
  }
}

// v[i][r] = w[i][r] / beta[r] (0 for a run whose beta is 0)
template <typename T, int VW>
__global__ void __launch_bounds__(kKmThreads) krylov_scale_kernel(const double* __restrict__ beta, int64_t n, int R,
                                                                 const typename Lane<T, VW>::type* __restrict__ w,
                                                                 typename Lane<T, VW>::type* __restrict__ v) {
  const int tpr = R / VW, rpb = kKmThreads / tpr;
  const int tid = threadIdx.x;
  const int c = tid % tpr, rr = tid / tpr;
  if (rr >= rpb) return;
  T inv[VW];
#pragma unroll
  for (int q = 0; q < VW; ++q) {
    const double b = beta[c * VW + q];
    inv[q] = b > 0.0 ? (T)(1.0 / b) : T(0);
  }
  // four row steps per iteration: their loads are issued before any store
  constexpr int U = 4;
  const int64_t step = (int64_t)gridDim.x * rpb;
  for (int64_t i0 = (int64_t)blockIdx.x * rpb + rr; i0 < n; i0 += U * step) {
    typename Lane<T, VW>::type a[U];
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (i0 + u * step < n) a[u] = __ldcs(w + (i0 + u * step) * tpr + c);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (i0 + u * step >= n) break;
      T re[VW], im[VW];
      unpack(a[u], re, im);
#pragma unroll
      for (int q = 0; q < VW; ++q) {
        re[q] *= inv[q];
        im[q] *= inv[q];
      }
      v[(i0 + u * step) * tpr + c] = pack(re, im);
    }
  }
}

inline int km_blocks(int64_t n, int R) {
  const int rpb = kKmThreads / R;
  int64_t b = (n + rpb - 1) / rpb;
  const int64_t cap = (int64_t)grid_cap() * 5;  // the projection's register limit: 5 blocks per SM
  if (b > cap) b = cap;
  return (int)(b > 0 ? b : 1);
}

inline bool a16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

template <typename T, int VW>
void launch_dot(dim3 grid, cudaStream_t s, const typename Lane<T, VW>::type* V, int64_t stride_l, int m, int64_t n,
                int R, const typename Lane<T, VW>::type* w, double2* partial) {
  constexpr size_t smem = dot_smem_bytes<T, VW>();
  // the ring is above the 48 KB default for 16-byte lanes (set on every call: per device)
  cudaFuncSetAttribute(krylov_dot_kernel<T, VW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  krylov_dot_kernel<T, VW><<<grid, kKmThreads, smem, s>>>(V, stride_l, m, n, R, w, partial);
}

// complex64 pairs per thread when every access of the call is a 16-byte one
inline bool pairs_ok(int R, int64_t stride, const void* a, const void* b) {
  return (R % 2) == 0 && (stride % 2) == 0 && a16(a) && a16(b);
}

}  // namespace
}  // namespace edgpu

using namespace edgpu;

extern "C" size_t edgpu_krylov_workspace(int64_t n, int R, int m_max) {
  if (n < 1 || R < 1 || R > kKmThreads || m_max < 1) return 0;
  const int nb = km_blocks(n, R);
  return sizeof(double2) * (size_t)m_max * nb * R + sizeof(double) * (size_t)nb * R + 512;
}

extern "C" int edgpu_krylov_dot(int precision, const void* V, int64_t stride, int m, int64_t n, int R, const void* w,
                                double* h, void* workspace, size_t workspace_bytes, void* stream) {
  if (!V || !w || !h || m < 1 || n < 1 || R < 1 || R > kKmThreads || stride < n * R) return EDGPU_ERR_ARG;
  if (precision != 0 && precision != 1) return EDGPU_ERR_ARG;
  if (workspace_bytes < edgpu_krylov_workspace(n, R, m)) return EDGPU_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  // row blocks: enough blocks for ~4 waves of 3 resident blocks per SM over all vector
  // groups, so that each block streams many row steps through its ring (its fill and its
  // reduction tree are paid once per block), at most the workspace's km_blocks
  const int ny = (m + KD - 1) / KD;
  const int nb = (int)std::min<int64_t>(km_blocks(n, R), std::max<int64_t>(1, ((int64_t)grid_cap() * 12 + ny - 1) / ny));
  double2* partial = reinterpret_cast<double2*>(workspace);
  dim3 grid(nb, ny);
  if (precision == 1 && pairs_ok(R, stride, V, w))
    launch_dot<float, 2>(grid, s, reinterpret_cast<const float4*>(V), stride / 2, m, n, R,
                         reinterpret_cast<const float4*>(w), partial);
  else if (precision == 1)
    launch_dot<float, 1>(grid, s, reinterpret_cast<const float2*>(V), stride, m, n, R,
                         reinterpret_cast<const float2*>(w), partial);
  else
    launch_dot<double, 1>(grid, s, reinterpret_cast<const double2*>(V), stride, m, n, R,
                          reinterpret_cast<const double2*>(w), partial);
  note_launch();
  krylov_dot_reduce_kernel<<<m, kKmThreads, 0, s>>>(partial, nb, R, reinterpret_cast<double2*>(h));
  note_launch();
  return check_launch();
}

extern "C" int edgpu_krylov_project(int precision, const void* V, int64_t stride, int m, int64_t n, int R,
                                    const double* h, void* w, int with_norm, void* workspace, size_t workspace_bytes,
                                    void* stream) {
  if (!V || !w || !h || m < 1 || n < 1 || R < 1 || R > kKmThreads || stride < n * R) return EDGPU_ERR_ARG;
  if (precision != 0 && precision != 1) return EDGPU_ERR_ARG;
  if (workspace_bytes < edgpu_krylov_workspace(n, R, 1)) return EDGPU_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = km_blocks(n, R);
  double* npart = with_norm ? reinterpret_cast<double*>(workspace) : nullptr;
  const double2* hc = reinterpret_cast<const double2*>(h);
  if (precision == 1 && pairs_ok(R, stride, V, w))
    krylov_project_kernel<float, 2><<<nb, kKmThreads, 0, s>>>(reinterpret_cast<const float4*>(V), stride / 2, m, n,
                                                              R, hc, reinterpret_cast<float4*>(w), npart);
  else if (precision == 1)
    krylov_project_kernel<float, 1><<<nb, kKmThreads, 0, s>>>(reinterpret_cast<const float2*>(V), stride, m, n, R,
                                                              hc, reinterpret_cast<float2*>(w), npart);
  else
    krylov_project_kernel<double, 1><<<nb, kKmThreads, 0, s>>>(reinterpret_cast<const double2*>(V), stride, m, n,
                                                               R, hc, reinterpret_cast<double2*>(w), npart);
  note_launch();
  return check_launch();
}

extern "C" int edgpu_krylov_normalize(int precision, int64_t n, int R, const void* w, void* v, double* beta,
                                      int32_t* status_dev, void* workspace, size_t workspace_bytes, void* stream) {
  if (!w || !v || !beta || n < 1 || R < 1 || R > kKmThreads) return EDGPU_ERR_ARG;
  if (precision != 0 && precision != 1) return EDGPU_ERR_ARG;
  if (workspace_bytes < edgpu_krylov_workspace(n, R, 1)) return EDGPU_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = km_blocks(n, R);
  const double* npart = reinterpret_cast<const double*>(workspace);
  krylov_norm_reduce_kernel<<<1, kKmThreads, 0, s>>>(npart, nb, R, beta, status_dev);
  note_launch();
  if (precision == 1 && pairs_ok(R, R, w, v))
    krylov_scale_kernel<float, 2><<<nb, kKmThreads, 0, s>>>(beta, n, R, reinterpret_cast<const float4*>(w),
                                                            reinterpret_cast<float4*>(v));
  else if (precision == 1)
    krylov_scale_kernel<float, 1><<<nb, kKmThreads, 0, s>>>(beta, n, R, reinterpret_cast<const float2*>(w),
                                                            reinterpret_cast<float2*>(v));
  else
    krylov_scale_kernel<double, 1><<<nb, kKmThreads, 0, s>>>(beta, n, R, reinterpret_cast<const double2*>(w),
                                                             reinterpret_cast<double2*>(v));
  note_launch();
  return check_launch();
}
