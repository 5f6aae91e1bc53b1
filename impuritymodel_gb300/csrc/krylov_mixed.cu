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
// Reductions: each thread sums its products over up to 8 rows in the vector type, then adds
// that partial into an FP64 accumulator; blocks reduce in shared memory in a fixed tree and a
// second launch adds the per-block partials in block order (deterministic, FP64 throughout
// above the first eight products).  Projections and scalings run in the vector type with the
// FP64 coefficients rounded to it.  All passes are bound by HBM reads of V.
#include "common.cuh"

namespace edgpu {
namespace {

template <typename T>
struct Cplx;
template <>
struct Cplx<float> {
  using type = float2;
};
template <>
struct Cplx<double> {
  using type = double2;
};

constexpr int kKmThreads = 256;
constexpr int kKmChunk = 8;  // products summed in the vector type before an FP64 add

inline int rows_per_block(int R) { return kKmThreads / R; }

// partial[k][b][r] = sum over this block's rows of conj(V[k][i][r]) * w[i][r], for the KD
// vectors k = blockIdx.y * KD + kk (w is read once for all of them)
constexpr int KD = 4;

template <typename T>
__global__ void __launch_bounds__(kKmThreads) krylov_dot_kernel(const typename Cplx<T>::type* __restrict__ V,
                                                               int64_t stride, int m, int64_t n, int R,
                                                               const typename Cplx<T>::type* __restrict__ w,
                                                               double2* __restrict__ partial) {
  using CT = typename Cplx<T>::type;
  __shared__ double2 red[kKmThreads];
  const int rpb = kKmThreads / R;
  const int tid = threadIdx.x;
  const int r = tid % R, rr = tid / R;
  const int k0 = blockIdx.y * KD;
  const int kn = m - k0 < KD ? m - k0 : KD;
  double sr[KD], si[KD];
#pragma unroll
  for (int kk = 0; kk < KD; ++kk) sr[kk] = si[kk] = 0.0;
  if (rr < rpb) {
    const int64_t step = (int64_t)gridDim.x * rpb;
    int64_t i = (int64_t)blockIdx.x * rpb + rr;
    while (i < n) {
      T cr[KD], ci[KD];
#pragma unroll
      for (int kk = 0; kk < KD; ++kk) cr[kk] = ci[kk] = T(0);
#pragma unroll 1
      for (int c = 0; c < kKmChunk; ++c) {
        if (i < n) {
          const CT b = w[i * R + r];
#pragma unroll
          for (int kk = 0; kk < KD; ++kk) {
            if (kk < kn) {
              const CT a = V[(int64_t)(k0 + kk) * stride + i * R + r];
              cr[kk] += a.x * b.x + a.y * b.y;
              ci[kk] += a.x * b.y - a.y * b.x;
            }
          }
        }
        i += step;
      }
#pragma unroll
      for (int kk = 0; kk < KD; ++kk) {
        sr[kk] += (double)cr[kk];
        si[kk] += (double)ci[kk];
      }
    }
  }
  for (int kk = 0; kk < kn; ++kk) {
    red[tid] = make_double2(sr[kk], si[kk]);
    __syncthreads();
    // rows of the block: fixed tree over rr for each r
    for (int h = (rpb + 1) / 2, len = rpb; len > 1; len = h, h = (h + 1) / 2) {
      if (rr < len - h && rr + h < len) {
        const double2 o = red[(rr + h) * R + r];
        red[tid].x += o.x;
        red[tid].y += o.y;
      }
      __syncthreads();
    }
    if (rr == 0) partial[((int64_t)(k0 + kk) * gridDim.x + blockIdx.x) * R + r] = red[r];
    __syncthreads();
  }
}

// h[k][r] = sum over blocks of partial[k][b][r] (block order)
__global__ void krylov_dot_reduce_kernel(const double2* __restrict__ partial, int nb, int m, int R, double2* h) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)m * R) return;
  const int k = (int)(t / R), r = (int)(t % R);
  double sr = 0.0, si = 0.0;
  for (int b = 0; b < nb; ++b) {
    const double2 p = partial[((int64_t)k * nb + b) * R + r];
    sr += p.x;
    si += p.y;
  }
  h[t] = make_double2(sr, si);
}

// w[i][r] -= sum_k h[k][r] V[k][i][r]; with norms: per-block FP64 partials of |w[.][r]|^2
template <typename T, int KB>
__global__ void __launch_bounds__(kKmThreads) krylov_project_kernel(const typename Cplx<T>::type* __restrict__ V,
                                                                   int64_t stride, int m, int64_t n, int R,
                                                                   const double2* __restrict__ h,
                                                                   typename Cplx<T>::type* __restrict__ w,
                                                                   double* __restrict__ npart) {
  using CT = typename Cplx<T>::type;
  __shared__ CT hs[KB];
  __shared__ double red[kKmThreads];
  const int rpb = kKmThreads / R;
  const int tid = threadIdx.x;
  const int r = tid % R, rr = tid / R;
  double nacc = 0.0;
  const int64_t step = (int64_t)gridDim.x * rpb;
  for (int k0 = 0; k0 < m; k0 += KB / R) {
    const int kc = (m - k0) < KB / R ? (m - k0) : KB / R;
    __syncthreads();
    for (int t = tid; t < kc * R; t += kKmThreads) {
      const double2 c = h[(int64_t)k0 * R + t];
      hs[t] = CT{(T)c.x, (T)c.y};
    }
    __syncthreads();
    if (rr < rpb) {
      for (int64_t i = (int64_t)blockIdx.x * rpb + rr; i < n; i += step) {
        CT acc = w[i * R + r];
        for (int k = 0; k < kc; ++k) {
          const CT c = hs[k * R + r];
          const CT v = V[(int64_t)(k0 + k) * stride + i * R + r];
          acc.x -= c.x * v.x - c.y * v.y;
          acc.y -= c.x * v.y + c.y * v.x;
        }
        w[i * R + r] = acc;
        if (npart && k0 + kc >= m) nacc += (double)acc.x * acc.x + (double)acc.y * acc.y;
      }
    }
  }
  if (!npart) return;
  red[tid] = nacc;
  __syncthreads();
  for (int hh = (rpb + 1) / 2, len = rpb; len > 1; len = hh, hh = (hh + 1) / 2) {
    if (rr < len - hh && rr + hh < len) red[tid] += red[(rr + hh) * R + r];
    __syncthreads();
  }
  if (rr == 0 && tid < R) npart[(int64_t)blockIdx.x * R + r] = red[r];
}

// beta[r] = sqrt(sum_b npart[b][r]); v[i][r] = w[i][r] / beta[r] (0 when beta[r] == 0, and
// the run's status flag set)
template <typename T>
__global__ void __launch_bounds__(kKmThreads) krylov_normalize_kernel(const double* __restrict__ npart, int nb,
                                                                     int64_t n, int R,
                                                                     const typename Cplx<T>::type* __restrict__ w,
                                                                     typename Cplx<T>::type* __restrict__ v,
                                                                     double* __restrict__ beta, int32_t* status) {
  using CT = typename Cplx<T>::type;
  __shared__ double sb[kKmThreads];
  const int tid = threadIdx.x;
  if (tid < R) {
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += npart[(int64_t)b * R + tid];
    sb[tid] = sqrt(s);
    if (blockIdx.x == 0) {
      beta[tid] = sb[tid];
      if (!(sb[tid] > 0.0) && status) atomicExch(status, (int32_t)EDGPU_ERR_BREAKDOWN);
    }
  }
  __syncthreads();
  const int rpb = kKmThreads / R;
  const int r = tid % R, rr = tid / R;
  if (rr >= rpb) return;
  const double b = sb[r];
  const T inv = b > 0.0 ? (T)(1.0 / b) : T(0);
  for (int64_t i = (int64_t)blockIdx.x * rpb + rr; i < n; i += (int64_t)gridDim.x * rpb) {
    const CT a = w[i * R + r];
    v[i * R + r] = CT{a.x * inv, a.y * inv};
  }
}

inline int km_blocks(int64_t n, int R) {
  const int rpb = rows_per_block(R);
  int64_t b = (n + rpb - 1) / rpb;
  const int64_t cap = (int64_t)grid_cap() * 4;
  if (b > cap) b = cap;
  return (int)(b > 0 ? b : 1);
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
  const int nb = km_blocks(n, R);
  double2* partial = reinterpret_cast<double2*>(workspace);
  dim3 grid(nb, (m + KD - 1) / KD);
  if (precision == 1)
    krylov_dot_kernel<float><<<grid, kKmThreads, 0, s>>>(reinterpret_cast<const float2*>(V), stride, m, n, R,
                                                         reinterpret_cast<const float2*>(w), partial);
  else
    krylov_dot_kernel<double><<<grid, kKmThreads, 0, s>>>(reinterpret_cast<const double2*>(V), stride, m, n, R,
                                                          reinterpret_cast<const double2*>(w), partial);
  note_launch();
  const int64_t t = (int64_t)m * R;
  krylov_dot_reduce_kernel<<<(unsigned)((t + 255) / 256), 256, 0, s>>>(partial, nb, m, R,
                                                                       reinterpret_cast<double2*>(h));
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
  constexpr int KB = 1024;  // coefficients staged per round (KB / R vectors)
  if (R > KB) return EDGPU_ERR_ARG;
  if (precision == 1)
    krylov_project_kernel<float, KB><<<nb, kKmThreads, 0, s>>>(reinterpret_cast<const float2*>(V), stride, m, n, R,
                                                               hc, reinterpret_cast<float2*>(w), npart);
  else
    krylov_project_kernel<double, KB><<<nb, kKmThreads, 0, s>>>(reinterpret_cast<const double2*>(V), stride, m, n,
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
  if (precision == 1)
    krylov_normalize_kernel<float><<<nb, kKmThreads, 0, s>>>(npart, nb, n, R, reinterpret_cast<const float2*>(w),
                                                             reinterpret_cast<float2*>(v), beta, status_dev);
  else
    krylov_normalize_kernel<double><<<nb, kKmThreads, 0, s>>>(npart, nb, n, R, reinterpret_cast<const double2*>(w),
                                                              reinterpret_cast<double2*>(v), beta, status_dev);
  note_launch();
  return check_launch();
}
