// Sparse H·v, batched Lanczos tridiagonalisation, Lanczos with full reorthogonalisation,
// Ritz/shifted-solve vector assembly and continued fractions.
//
// Upstream counterparts: get_tridiagonal_krylov_vectors (impurityModel/ed/finite.py:1897-1995),
// scipy eigsh in eigensystem (finite.py:105), BiCGSTAB in getRIXSmap (spectra.py:962,1080)
// and the continued fraction of getGreen (spectra.py:678-680).
//
// Vectors of a batch are stored [n][R] (run index fastest) so that the R threads of one
// row read the row's CSR entries once (broadcast) and gather x[col][0..R) contiguously.
// All reductions are deterministic: per-block partials in fixed order, summed in fixed order.
#include <algorithm>
#include <atomic>
#include <vector>

#include "common.cuh"
#include "df64.cuh"

namespace edgpu {

template <typename T>
struct Cx;
template <>
struct Cx<double> {
  using V = double2;
};
template <>
struct Cx<float> {
  using V = float2;
};

__device__ __forceinline__ double2 ld(const double2* p) { return *p; }
__device__ __forceinline__ float2 ld(const float2* p) { return *p; }

struct RunTile {
  int rt;   // runs per block (blockDim.x)
  int rb;   // rows per block pass (blockDim.y)
  int nrb;  // row blocks (gridDim.x)
  int nrt;  // run tiles (gridDim.y)
};

inline RunTile make_tile(int64_t n, int R) {
  RunTile t;
  t.rt = R < 32 ? R : 32;
  t.rb = 256 / t.rt;
  if (t.rb < 1) t.rb = 1;
  t.nrt = (R + t.rt - 1) / t.rt;
  int64_t nrb = (n + t.rb - 1) / t.rb;
  // about 4 blocks per SM in total over the (row block, run tile) grid
  int64_t cap = ((int64_t)grid_cap() * 4 + t.nrt - 1) / t.nrt;
  if (cap < 1) cap = 1;
  if (nrb > cap) nrb = cap;
  if (nrb < 1) nrb = 1;
  t.nrb = (int)nrb;
  return t;
}

// Y = H X and alpha partial Re<Y, X> per run.  T: vector/accumulation scalar, VALC: complex values.
template <typename T, bool VALC>
__global__ void spmm_alpha_kernel(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                  const T* __restrict__ vals, int R, const typename Cx<T>::V* __restrict__ X,
                                  typename Cx<T>::V* __restrict__ Y, double* __restrict__ partial, int with_alpha) {
  using V = typename Cx<T>::V;
  extern __shared__ double red[];
  const int tr = threadIdx.x, ti = threadIdx.y;
  const int r = blockIdx.y * blockDim.x + tr;
  double acc = 0.0;
  if (r < R) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.y + ti; i < n; i += (int64_t)gridDim.x * blockDim.y) {
      T yr = 0, yi = 0;
      const int64_t e1 = rp[i + 1];
      for (int64_t e = rp[i]; e < e1; ++e) {
        const int c = col[e];
        const V x = ld(X + (int64_t)c * R + r);
        if (VALC) {
          const T hr = vals[2 * e], hi = vals[2 * e + 1];
          yr += hr * x.x - hi * x.y;
          yi += hr * x.y + hi * x.x;
        } else {
          const T h = vals[e];
          yr += h * x.x;
          yi += h * x.y;
        }
      }
      V y;
      y.x = yr;
      y.y = yi;
      Y[i * R + r] = y;
      if (with_alpha) {
        const V v = ld(X + i * R + r);
        acc += (double)yr * (double)v.x + (double)yi * (double)v.y;
      }
    }
  }
  if (!with_alpha) return;
  red[ti * blockDim.x + tr] = acc;
  __syncthreads();
  if (ti == 0 && r < R) {
    double s = 0.0;
    for (int k = 0; k < (int)blockDim.y; ++k) s += red[k * blockDim.x + tr];
    partial[(int64_t)blockIdx.x * R + r] = s;
  }
}

// alpha_r = sum of partials; W = Y - alpha Vc - beta_prev Vp; beta partial ||W||^2.
template <typename T>
__global__ void axpy_beta_kernel(int64_t n, int R, typename Cx<T>::V* __restrict__ Y,
                                 const typename Cx<T>::V* __restrict__ Vc, const typename Cx<T>::V* __restrict__ Vp,
                                 const double* __restrict__ palpha, int nrb, const double* __restrict__ beta_prev,
                                 double* __restrict__ alpha_out, int K, int j, double* __restrict__ pbeta) {
  using V = typename Cx<T>::V;
  extern __shared__ double red[];
  __shared__ double alpha_s[32];
  const int tr = threadIdx.x, ti = threadIdx.y;
  const int r = blockIdx.y * blockDim.x + tr;
  if (ti == 0 && r < R) {
    double a = 0.0;
    for (int b = 0; b < nrb; ++b) a += palpha[(int64_t)b * R + r];
    alpha_s[tr] = a;
    if (blockIdx.x == 0) alpha_out[(int64_t)r * K + j] = a;
  }
  __syncthreads();
  double acc = 0.0;
  if (r < R) {
    const double a = alpha_s[tr];
    const double bp = beta_prev ? beta_prev[(int64_t)r * K + (j - 1)] : 0.0;
    const T af = (T)a, bf = (T)bp;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.y + ti; i < n; i += (int64_t)gridDim.x * blockDim.y) {
      V y = Y[i * R + r];
      const V c = ld(Vc + i * R + r);
      y.x -= af * c.x;
      y.y -= af * c.y;
      if (Vp) {
        const V p = ld(Vp + i * R + r);
        y.x -= bf * p.x;
        y.y -= bf * p.y;
      }
      Y[i * R + r] = y;
      acc += (double)y.x * (double)y.x + (double)y.y * (double)y.y;
    }
  }
  red[ti * blockDim.x + tr] = acc;
  __syncthreads();
  if (ti == 0 && r < R) {
    double s = 0.0;
    for (int k = 0; k < (int)blockDim.y; ++k) s += red[k * blockDim.x + tr];
    pbeta[(int64_t)blockIdx.x * R + r] = s;
  }
}

// beta_r = sqrt(sum partials); Vn = W / beta.
template <typename T>
__global__ void normalize_kernel(int64_t n, int R, const typename Cx<T>::V* __restrict__ Wv,
                                 typename Cx<T>::V* __restrict__ Vn, const double* __restrict__ pbeta, int nrb,
                                 double* __restrict__ beta_out, int K, int j, const int32_t* __restrict__ k_max,
                                 int32_t* status) {
  using V = typename Cx<T>::V;
  __shared__ double beta_s[32];
  const int tr = threadIdx.x, ti = threadIdx.y;
  const int r = blockIdx.y * blockDim.x + tr;
  if (ti == 0 && r < R) {
    double s = 0.0;
    for (int b = 0; b < nrb; ++b) s += pbeta[(int64_t)b * R + r];
    const double bt = sqrt(s);
    beta_s[tr] = bt;
    if (blockIdx.x == 0) {
      beta_out[(int64_t)r * K + j] = bt;
      if (k_max[r] > j + 1 && !(bt > 0.0))
        atomicExch(status, (int32_t)(bt == 0.0 ? EDGPU_ERR_BREAKDOWN : EDGPU_ERR_NAN));
    }
  }
  __syncthreads();
  if (r >= R) return;
  const double beta = beta_s[tr];
  const T inv = beta > 0.0 ? (T)(1.0 / beta) : (T)0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.y + ti; i < n; i += (int64_t)gridDim.x * blockDim.y) {
    V w = Wv[i * R + r];
    V o;
    // one reciprocal per run and step: FP64 division is many times the cost of an FMA
    o.x = w.x * inv;
    o.y = w.y * inv;
    Vn[i * R + r] = o;
  }
}

__global__ void to_c64_kernel(const double2* in, float2* out, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = in[i];
    out[i] = make_float2((float)v.x, (float)v.y);
  }
}

__global__ void copy_c128_kernel(const double2* in, double2* out, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = in[i];
}

// ---------------------------------------------------------------------------------------
// Full reorthogonalisation: dots h[k] = <V_k, w>, k < m; then w -= sum_k h[k] V_k.
// ---------------------------------------------------------------------------------------
constexpr int kDotTile = 8;

__global__ void multidot_kernel(const double2* __restrict__ V, int m, int64_t n, const double2* __restrict__ w,
                                double2* __restrict__ partial) {
  __shared__ double2 red[kDotTile][256 / 32];
  const int k0 = blockIdx.y * kDotTile;
  double2 acc[kDotTile];
#pragma unroll
  for (int k = 0; k < kDotTile; ++k) acc[k] = make_double2(0.0, 0.0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 x = w[i];
#pragma unroll
    for (int k = 0; k < kDotTile; ++k) {
      if (k0 + k < m) {
        const double2 v = V[(int64_t)(k0 + k) * n + i];
        acc[k].x += v.x * x.x + v.y * x.y;
        acc[k].y += v.x * x.y - v.y * x.x;
      }
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kDotTile; ++k) {
    double a = acc[k].x, b = acc[k].y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) red[k][warp] = make_double2(a, b);
  }
  __syncthreads();
  if (threadIdx.x < kDotTile && k0 + threadIdx.x < m) {
    double a = 0.0, b = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
      a += red[threadIdx.x][q].x;
      b += red[threadIdx.x][q].y;
    }
    partial[(int64_t)(k0 + threadIdx.x) * gridDim.x + blockIdx.x] = make_double2(a, b);
  }
}

__global__ void sum_partials_kernel(const double2* partial, int m, int nb, double2* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  double a = 0.0, b = 0.0;
  for (int q = 0; q < nb; ++q) {
    a += partial[(int64_t)k * nb + q].x;
    b += partial[(int64_t)k * nb + q].y;
  }
  out[k] = make_double2(a, b);
}

__global__ void subtract_proj_kernel(const double2* __restrict__ V, int m, int64_t n, const double2* __restrict__ h,
                                     double2* __restrict__ w) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double2 x = w[i];
#pragma unroll 8
    for (int k = 0; k < m; ++k) {
      const double2 c = h[k];
      const double2 v = V[(int64_t)k * n + i];
      x.x -= c.x * v.x - c.y * v.y;
      x.y -= c.x * v.y + c.y * v.x;
    }
    w[i] = x;
  }
}

// Single-run helpers for the reorthogonalised Lanczos (R == 1 specialisations).
__global__ void reorth_alpha_update_kernel(int64_t n, double2* w, const double2* vj, const double2* vjm1,
                                           const double* palpha, int nrb, double* alpha, const double* beta, int j,
                                           double* pnorm) {
  __shared__ double red[256];
  __shared__ double a_s;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int b = 0; b < nrb; ++b) t += palpha[b];
    a_s = t;
    if (blockIdx.x == 0) alpha[j] = t;
  }
  __syncthreads();
  const double a = a_s;
  const double bp = (j > 0) ? beta[j - 1] : 0.0;
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double2 y = w[i];
    const double2 c = vj[i];
    y.x -= a * c.x;
    y.y -= a * c.y;
    if (j > 0) {
      const double2 p = vjm1[i];
      y.x -= bp * p.x;
      y.y -= bp * p.y;
    }
    w[i] = y;
    acc += y.x * y.x + y.y * y.y;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)blockDim.x; ++k) s += red[k];
    pnorm[blockIdx.x] = s;
  }
}

// h[k] = <V_k, w> for k < m: one block per k, whole vector, deterministic block tree.
__global__ void __launch_bounds__(256) dot_per_k_kernel(const double2* __restrict__ V, int m, int64_t n,
                                                        const double2* __restrict__ w, double2* __restrict__ h) {
  __shared__ double red_r[8], red_i[8];
  const int k = blockIdx.x;
  if (k >= m) return;
  const double2* vk = V + (int64_t)k * n;
  double hr = 0.0, hi = 0.0;
#pragma unroll 4
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double2 v = vk[i], x = w[i];
    hr += v.x * x.x + v.y * x.y;
    hi += v.x * x.y - v.y * x.x;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    hr += __shfl_down_sync(0xffffffffu, hr, o);
    hi += __shfl_down_sync(0xffffffffu, hi, o);
  }
  if (lane == 0) {
    red_r[warp] = hr;
    red_i[warp] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
      a += red_r[q];
      b += red_i[q];
    }
    h[k] = make_double2(a, b);
  }
}

// w -= sum_k h[k] V_k, block = 32 rows x 8 k-residue classes (smem reduction over the 8);
// with_norm: per-block partial |w|^2 of the updated rows into pnorm[blockIdx.x].
__global__ void __launch_bounds__(256) project_out_kernel(const double2* __restrict__ V, int m, int64_t n,
                                                          const double2* __restrict__ h, double2* __restrict__ w,
                                                          double* __restrict__ pnorm, int with_norm) {
  __shared__ double2 part[8][32];
  __shared__ double nrm[32];
  const int ri = threadIdx.x & 31, kc = threadIdx.x >> 5;
  const int64_t i = (int64_t)blockIdx.x * 32 + ri;
  double2 acc = make_double2(0.0, 0.0);
  if (i < n) {
#pragma unroll 4
    for (int k = kc; k < m; k += 8) {
      const double2 c = h[k];
      const double2 v = V[(int64_t)k * n + i];
      acc.x += c.x * v.x - c.y * v.y;
      acc.y += c.x * v.y + c.y * v.x;
    }
  }
  part[kc][ri] = acc;
  __syncthreads();
  if (kc == 0) {
    double nr = 0.0;
    if (i < n) {
      double2 x = w[i];
      for (int q = 0; q < 8; ++q) {
        x.x -= part[q][ri].x;
        x.y -= part[q][ri].y;
      }
      w[i] = x;
      nr = x.x * x.x + x.y * x.y;
    }
    nrm[ri] = nr;
  }
  __syncthreads();
  if (with_norm && threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < 32; ++q) t += nrm[q];
    pnorm[blockIdx.x] = t;
  }
}

__global__ void norm_partial_kernel(int64_t n, const double2* w, double* pnorm) {
  __shared__ double red[256];
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 y = w[i];
    acc += y.x * y.x + y.y * y.y;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)blockDim.x; ++k) s += red[k];
    pnorm[blockIdx.x] = s;
  }
}

__global__ void reorth_normalize_kernel(int64_t n, const double2* w, double2* vnext, const double* pnorm, int nb,
                                        double* beta, int j, int32_t* status) {
  __shared__ double bt_s;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += pnorm[b];
    bt_s = sqrt(s);
    if (blockIdx.x == 0) {
      beta[j] = bt_s;
      if (!(bt_s > 0.0)) atomicExch(status, (int32_t)(bt_s == 0.0 ? EDGPU_ERR_BREAKDOWN : EDGPU_ERR_NAN));
    }
  }
  __syncthreads();
  const double bt = bt_s;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 y = w[i];
    vnext[i] = bt > 0.0 ? make_double2(y.x / bt, y.y / bt) : make_double2(0.0, 0.0);
  }
}

// X[m][i] = sum_k C[k][m] V[k][i]
__global__ void combine_kernel(const double2* __restrict__ V, int K, int64_t n, const double2* __restrict__ C, int M,
                               double2* __restrict__ X) {
  const int m = blockIdx.y;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double xr = 0.0, xi = 0.0;
#pragma unroll 8
    for (int k = 0; k < K; ++k) {
      const double2 c = C[(int64_t)k * M + m];
      const double2 v = V[(int64_t)k * n + i];
      xr += c.x * v.x - c.y * v.y;
      xi += c.x * v.y + c.y * v.x;
    }
    X[(int64_t)m * n + i] = make_double2(xr, xi);
  }
}

// Continued fraction, thread per (run, omega).
__global__ void cfrac_kernel(const double* __restrict__ alpha, const double* __restrict__ beta,
                             const int32_t* __restrict__ k_len, int K, int R, const double* __restrict__ omega,
                             int n_omega, double delta, const double* __restrict__ e, const double* __restrict__ scale,
                             double2* __restrict__ g) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (int64_t)R * n_omega) return;
  const int r = (int)(tid / n_omega);
  const int w = (int)(tid % n_omega);
  const int kl = k_len[r];
  const double zr = omega[w] + e[r];
  const double zi = delta;
  double gr = 0.0, gi = 0.0;
  const double* a = alpha + (int64_t)r * K;
  const double* b = beta + (int64_t)r * K;
  for (int i = kl - 1; i >= 0; --i) {
    double dr = zr - a[i];
    double di = zi;
    if (i != kl - 1) {
      const double b2 = b[i] * b[i];
      dr -= b2 * gr;
      di -= b2 * gi;
    }
    // g = 1 / (dr + i di) = (dr - i di) / |d|^2; |d| >= delta > 0 and the entries are
    // energies of order 1e3 eV at most, so |d|^2 neither overflows nor underflows
    const double inv = 1.0 / (dr * dr + di * di);
    gr = dr * inv;
    gi = -di * inv;
  }
  const double s = scale ? scale[r] : 1.0;
  g[tid] = kl > 0 ? make_double2(s * gr, s * gi) : make_double2(0.0, 0.0);
}

bool small_fits(int64_t n, int precision);
int lanczos_small(const edgpu_csr* h, const double* v0, int R, const int32_t* k_max, int K, int precision,
                  double* alpha, double* beta, int32_t* status, void* ws, cudaStream_t s);

// Mixed form: a'[r][i] = float(alpha - e_r), b2[r][i] = float(beta^2) (FP64 subtraction
// first, so the large common energy cancels exactly), then the fraction in float32.
__global__ void cfrac_prep_kernel(const double* __restrict__ alpha, const double* __restrict__ beta,
                                  const int32_t* __restrict__ k_len, int K, int R, const double* __restrict__ e,
                                  float* __restrict__ ap, float* __restrict__ b2) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)R * K) return;
  const int r = (int)(t / K);
  ap[t] = (float)(alpha[t] - e[r]);
  b2[t] = (float)(beta[t] * beta[t]);
  (void)k_len;
}

__global__ void cfrac_f32_kernel(const float* __restrict__ ap, const float* __restrict__ b2,
                                 const int32_t* __restrict__ k_len, int K, int R, const double* __restrict__ omega,
                                 int n_omega, double delta, const double* __restrict__ scale, double2* __restrict__ g) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (int64_t)R * n_omega) return;
  const int r = (int)(tid / n_omega);
  const int w = (int)(tid % n_omega);
  const int kl = k_len[r];
  const float zr = (float)omega[w];
  const float zi = (float)delta;
  const float* a = ap + (int64_t)r * K;
  const float* b = b2 + (int64_t)r * K;
  float gr = 0.f, gi = 0.f;
  for (int i = kl - 1; i >= 0; --i) {
    float dr = zr - a[i], di = zi;
    if (i != kl - 1) {
      dr -= b[i] * gr;
      di -= b[i] * gi;
    }
    const float inv = 1.0f / (dr * dr + di * di);
    gr = dr * inv;
    gi = -di * inv;
  }
  const double s = scale ? scale[r] : 1.0;
  g[tid] = kl > 0 ? make_double2(s * (double)gr, s * (double)gi) : make_double2(0.0, 0.0);
}

inline unsigned grid_1d(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)grid_cap() * 8;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

// Row-parallel SpMM for y = H x with x, y [n][R]: thread = (row i, group g of RV runs),
// L = R / RV threads per row, one row per thread, 16-byte vector loads of x (float4 holds
// two complex64 runs, double2 one complex128 run) and UNROLL independent gathers in flight.
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
  static constexpr int runs = 2;
};
template <>
struct Vec16<double> {
  using type = double2;
  static constexpr int runs = 1;
};

constexpr int kRowsThreads = 128;  // smaller blocks shorten the tail of ragged rows

template <typename T, bool VALC>
__global__ void __launch_bounds__(kRowsThreads) spmm_rows_kernel(int64_t n, const int64_t* __restrict__ rp,
                                                                 const int32_t* __restrict__ col,
                                                                 const T* __restrict__ vals, int R, int L,
                                                                 const typename Cx<T>::V* __restrict__ X,
                                                                 typename Cx<T>::V* __restrict__ Y) {
  using Q = typename Vec16<T>::type;
  constexpr int RV = Vec16<T>::runs;
  constexpr int UNROLL = 8;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i = gt / L;
  const int g = (int)(gt - i * L);
  if (i >= n) return;
  const int64_t r0 = (int64_t)g * RV;
  T ar[RV], ai[RV];
#pragma unroll
  for (int q = 0; q < RV; ++q) ar[q] = ai[q] = 0;
  const int64_t e1 = __ldg(rp + i + 1);
  // Batches of UNROLL entries, the last one predicated: every row needs at most three
  // dependent memory round trips per batch (row pointers, CSR entries, gathers of x).
  for (int64_t e = __ldg(rp + i); e < e1; e += UNROLL) {
    int c[UNROLL];
    T hr[UNROLL], hi[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      const bool ok = e + u < e1;
      // CSR entries are read once: streaming loads keep x resident in L2
      c[u] = ok ? __ldcs(col + e + u) : 0;
      if (VALC) {
        hr[u] = ok ? __ldcs(vals + 2 * (e + u)) : T(0);
        hi[u] = ok ? __ldcs(vals + 2 * (e + u) + 1) : T(0);
      } else {
        hr[u] = ok ? __ldcs(vals + e + u) : T(0);
        hi[u] = 0;
      }
    }
    Q xv[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; ++u)
      xv[u] = (e + u < e1) ? __ldg(reinterpret_cast<const Q*>(X + (int64_t)c[u] * R + r0)) : Q{};
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
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
  Q out;
  T* os = reinterpret_cast<T*>(&out);
#pragma unroll
  for (int q = 0; q < RV; ++q) {
    os[2 * q] = ar[q];
    os[2 * q + 1] = ai[q];
  }
  __stcs(reinterpret_cast<Q*>(Y + i * R + r0), out);
}

template <typename T>
int spmv_impl(const edgpu_csr* h, const typename Cx<T>::V* x, typename Cx<T>::V* y, int R, cudaStream_t s) {
  constexpr int RV = Vec16<T>::runs;
  if (R % RV == 0) {
    const int L = R / RV;
    const int64_t threads = h->n * (int64_t)L;
    const unsigned blocks = (unsigned)((threads + kRowsThreads - 1) / kRowsThreads);
    const int bt = kRowsThreads;
    if (sizeof(T) == 8) {
      if (h->val_c)
        spmm_rows_kernel<T, true><<<blocks, bt, 0, s>>>(h->n, h->row_ptr, h->col, (const T*)h->val_c, R, L, x, y);
      else
        spmm_rows_kernel<T, false><<<blocks, bt, 0, s>>>(h->n, h->row_ptr, h->col, (const T*)h->val_r, R, L, x, y);
    } else {
      if (h->val_cf)
        spmm_rows_kernel<T, true><<<blocks, bt, 0, s>>>(h->n, h->row_ptr, h->col, (const T*)h->val_cf, R, L, x, y);
      else
        spmm_rows_kernel<T, false><<<blocks, bt, 0, s>>>(h->n, h->row_ptr, h->col, (const T*)h->val_rf, R, L, x, y);
    }
    note_launch();
    return check_launch();
  }
  RunTile t = make_tile(h->n, R);
  dim3 grid(t.nrb, t.nrt), block(t.rt, t.rb);
  if (sizeof(T) == 8) {
    if (h->val_c)
      spmm_alpha_kernel<T, true><<<grid, block, 0, s>>>(h->n, h->row_ptr, h->col, (const T*)h->val_c, R,
                                                        x, y, nullptr, 0);
    else
      spmm_alpha_kernel<T, false><<<grid, block, 0, s>>>(h->n, h->row_ptr, h->col, (const T*)h->val_r, R,
                                                         x, y, nullptr, 0); note_launch();
  } else {
    if (h->val_cf)
      spmm_alpha_kernel<T, true><<<grid, block, 0, s>>>(h->n, h->row_ptr, h->col, (const T*)h->val_cf, R,
                                                        x, y, nullptr, 0);
    else
      spmm_alpha_kernel<T, false><<<grid, block, 0, s>>>(h->n, h->row_ptr, h->col, (const T*)h->val_rf, R,
                                                         x, y, nullptr, 0); note_launch();
  }
  return check_launch();
}

// Optional per-kernel timing with CUDA events on the launching stream: kernel_ms[0..2] receive
// the summed durations of the SpMM, axpy/beta and normalise launches (host array).
struct KernelTimer {
  double* out;
  std::vector<cudaEvent_t> ev[3];
  cudaStream_t s;
  KernelTimer(double* o, int K, cudaStream_t st) : out(o), s(st) {
    if (!out) return;
    for (int k = 0; k < 3; ++k) {
      ev[k].resize(2 * (size_t)K);
      for (auto& e : ev[k]) cudaEventCreate(&e);
    }
  }
  void mark(int kind, int j, int phase) {
    if (out) cudaEventRecord(ev[kind][2 * (size_t)j + phase], s);
  }
  void finish(int K) {
    if (!out) return;
    for (int k = 0; k < 3; ++k) {
      double tot = 0.0;
      for (int j = 0; j < K; ++j) {
        if (k == 2 && j == K - 1) continue;
        float ms = 0.f;
        cudaEventSynchronize(ev[k][2 * (size_t)j + 1]);
        if (cudaEventElapsedTime(&ms, ev[k][2 * (size_t)j], ev[k][2 * (size_t)j + 1]) == cudaSuccess) tot += ms;
      }
      out[k] = tot;
    }
    for (int k = 0; k < 3; ++k)
      for (auto& e : ev[k]) cudaEventDestroy(e);
  }
};

template <typename T>
int lanczos_impl(const edgpu_csr* h, const double* v0, int R, const int32_t* k_max, int K, double* alpha, double* beta,
                 int32_t* status, unsigned char* ws, size_t ws_bytes, cudaStream_t s, double* kernel_ms = nullptr) {
  using V = typename Cx<T>::V;
  const int64_t n = h->n;
  const int64_t nv = n * (int64_t)R;
  RunTile t = make_tile(n, R);
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    unsigned char* p = ws + off;
    off += (bytes + 255) & ~(size_t)255;
    return p;
  };
  V* A = reinterpret_cast<V*>(carve(sizeof(V) * nv));
  V* B = reinterpret_cast<V*>(carve(sizeof(V) * nv));
  V* Wb = reinterpret_cast<V*>(carve(sizeof(V) * nv));
  double* pa = reinterpret_cast<double*>(carve(sizeof(double) * (size_t)t.nrb * R));
  double* pb = reinterpret_cast<double*>(carve(sizeof(double) * (size_t)t.nrb * R));
  if (off > ws_bytes) return EDGPU_ERR_WORKSPACE;
  if (sizeof(T) == 8)
    copy_c128_kernel<<<grid_1d(nv, 256), 256, 0, s>>>(reinterpret_cast<const double2*>(v0),
                                                       reinterpret_cast<double2*>(A), nv);
  else
    to_c64_kernel<<<grid_1d(nv, 256), 256, 0, s>>>(reinterpret_cast<const double2*>(v0),
                                                    reinterpret_cast<float2*>(A), nv); note_launch();
  int rc = check_launch();
  if (rc) return rc;
  dim3 grid(t.nrb, t.nrt), block(t.rt, t.rb);
  const size_t red = sizeof(double) * (size_t)t.rt * t.rb;
  const T* vals = nullptr;
  bool valc = false;
  if (sizeof(T) == 8) {
    valc = h->val_c != nullptr;
    vals = (const T*)(valc ? (const void*)h->val_c : (const void*)h->val_r);
  } else {
    valc = h->val_cf != nullptr;
    vals = (const T*)(valc ? (const void*)h->val_cf : (const void*)h->val_rf);
  }
  if (!vals) return EDGPU_ERR_ARG;
  V* Vc = A;
  V* Vp = B;
  KernelTimer timer(kernel_ms, K, s);
  for (int j = 0; j < K; ++j) {
    timer.mark(0, j, 0);
    if (valc)
      spmm_alpha_kernel<T, true><<<grid, block, red, s>>>(n, h->row_ptr, h->col, vals, R, Vc, Wb, pa, 1);
    else
      spmm_alpha_kernel<T, false><<<grid, block, red, s>>>(n, h->row_ptr, h->col, vals, R, Vc, Wb, pa, 1); note_launch();
    timer.mark(0, j, 1);
    timer.mark(1, j, 0);
    axpy_beta_kernel<T><<<grid, block, red, s>>>(n, R, Wb, Vc, j > 0 ? Vp : nullptr, pa, t.nrb,
                                                 j > 0 ? beta : nullptr, alpha, K, j, pb); note_launch();
    timer.mark(1, j, 1);
    if (j + 1 < K) {
      timer.mark(2, j, 0);
      normalize_kernel<T><<<grid, block, 0, s>>>(n, R, Wb, Vp, pb, t.nrb, beta, K, j, k_max, status);
      note_launch();
      timer.mark(2, j, 1);
    }
    if ((rc = check_launch())) return rc;
    V* tmp = Vc;
    Vc = Vp;
    Vp = tmp;
  }
  timer.finish(K);
  return EDGPU_OK;
}

}  // namespace edgpu

using namespace edgpu;

extern "C" int edgpu_spmv(const edgpu_csr* h, const double* x, double* y, int R, void* stream) {
  if (!h || !x || !y || R < 1 || h->n < 0) return EDGPU_ERR_ARG;
  if (!h->val_c && !h->val_r) return EDGPU_ERR_ARG;
  if (h->n == 0) return EDGPU_OK;
  return spmv_impl<double>(h, reinterpret_cast<const double2*>(x), reinterpret_cast<double2*>(y), R,
                           (cudaStream_t)stream);
}

extern "C" int edgpu_spmv_c64(const edgpu_csr* h, const float* x, float* y, int R, void* stream) {
  if (!h || !x || !y || R < 1 || h->n < 0) return EDGPU_ERR_ARG;
  if (!h->val_cf && !h->val_rf) return EDGPU_ERR_ARG;
  if (h->n == 0) return EDGPU_OK;
  return spmv_impl<float>(h, reinterpret_cast<const float2*>(x), reinterpret_cast<float2*>(y), R,
                          (cudaStream_t)stream);
}

extern "C" size_t edgpu_lanczos_workspace(int64_t n, int R, int K, int precision) {
  (void)K;
  const size_t vs = precision == 1 ? sizeof(float2) : sizeof(double2);
  RunTile t = make_tile(n > 0 ? n : 1, R > 0 ? R : 1);
  size_t b = 0;
  for (int k = 0; k < 3; ++k) b += ((vs * (size_t)n * R) + 255) & ~(size_t)255;
  b += 2 * (((sizeof(double) * (size_t)t.nrb * R) + 255) & ~(size_t)255);
  return b + 256;
}

// The df64 form (precision 3) exists for real H in the shared-memory path; everything else
// it asks for runs in FP64.
static int effective_precision(const edgpu_csr* h, int precision) {
  if (precision != 3) return precision;
  return (h->val_df && !h->val_c && small_fits(h->n, 3)) ? 3 : 0;
}

extern "C" int edgpu_lanczos(const edgpu_csr* h, const double* v0, int R, const int32_t* k_max, int K, int precision,
                             double* alpha, double* beta, int32_t* status_dev, void* workspace, size_t workspace_bytes,
                             void* stream) {
  if (!h || !v0 || R < 1 || K < 1 || !k_max || !alpha || !beta || !status_dev || h->n < 1) return EDGPU_ERR_ARG;
  if (precision < 0 || precision > 3 || precision == 2) return EDGPU_ERR_ARG;
  precision = effective_precision(h, precision);
  if (workspace_bytes < edgpu_lanczos_workspace(h->n, R, K, precision)) return EDGPU_ERR_WORKSPACE;
  unsigned char* ws = reinterpret_cast<unsigned char*>(workspace);
  if (small_fits(h->n, precision))
    return lanczos_small(h, v0, R, k_max, K, precision, alpha, beta, status_dev, ws, (cudaStream_t)stream);
  if (precision == 0)
    return lanczos_impl<double>(h, v0, R, k_max, K, alpha, beta, status_dev, ws, workspace_bytes,
                                (cudaStream_t)stream);
  return lanczos_impl<float>(h, v0, R, k_max, K, alpha, beta, status_dev, ws, workspace_bytes, (cudaStream_t)stream);
}

extern "C" int edgpu_lanczos_timed(const edgpu_csr* h, const double* v0, int R, const int32_t* k_max, int K,
                                   int precision, double* alpha, double* beta, int32_t* status_dev, void* workspace,
                                   size_t workspace_bytes, void* stream, double* kernel_ms) {
  if (!h || !v0 || R < 1 || K < 1 || !k_max || !alpha || !beta || !status_dev || h->n < 1 || !kernel_ms)
    return EDGPU_ERR_ARG;
  if (precision < 0 || precision > 3 || precision == 2) return EDGPU_ERR_ARG;
  precision = effective_precision(h, precision);
  if (workspace_bytes < edgpu_lanczos_workspace(h->n, R, K, precision)) return EDGPU_ERR_WORKSPACE;
  unsigned char* ws = reinterpret_cast<unsigned char*>(workspace);
  if (small_fits(h->n, precision)) {
    cudaStream_t s = (cudaStream_t)stream;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    int rc = lanczos_small(h, v0, R, k_max, K, precision, alpha, beta, status_dev, ws, s);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    kernel_ms[0] = ms;  // whole fused Krylov loop (SpMV, reductions, axpy) in one launch
    kernel_ms[1] = 0.0;
    kernel_ms[2] = 0.0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
  }
  if (precision == 0)
    return lanczos_impl<double>(h, v0, R, k_max, K, alpha, beta, status_dev, ws, workspace_bytes,
                                (cudaStream_t)stream, kernel_ms);
  return lanczos_impl<float>(h, v0, R, k_max, K, alpha, beta, status_dev, ws, workspace_bytes, (cudaStream_t)stream,
                             kernel_ms);
}

namespace edgpu {
size_t reorth_coop_scratch_bytes();
int lanczos_reorth_coop(const edgpu_csr* h, const double* v0, int j0, int j1, int K_cap, double* Vd, double* wd,
                        double* alpha, double* beta, int32_t* status_dev, double* scratch, double2* hc,
                        cudaStream_t s);
}  // namespace edgpu
static std::atomic<int> g_reorth_fused{1};

extern "C" void edgpu_set_reorth_fused(int enabled) { g_reorth_fused.store(enabled ? 1 : 0); }

extern "C" size_t edgpu_lanczos_reorth_workspace(int64_t n, int K_cap) {
  const int64_t nrb = grid_1d(n > 0 ? n : 1, 256);
  size_t b = 0;
  b += sizeof(double2) * (size_t)n;                        // y
  b += sizeof(double) * (size_t)nrb * 2 + 512;             // alpha/norm partials
  b += sizeof(double2) * (size_t)(K_cap + 1) * nrb + 256;  // dot partials
  b += sizeof(double2) * (size_t)(K_cap + 1) + 256;        // h
  b += sizeof(double) * (size_t)((n + 31) / 32 + 1) + 256;  // projection-block norm partials
  b += reorth_coop_scratch_bytes() + 256;                   // per-block partials of the fused form
  return b + 1024;
}


extern "C" int edgpu_lanczos_reorth(const edgpu_csr* h, const double* v0, int j0, int j1, int K_cap, double* Vd,
                                    double* wd, double* alpha, double* beta, int32_t* status_dev, void* workspace,
                                    size_t workspace_bytes, void* stream) {
  if (!h || !Vd || !wd || !alpha || !beta || !status_dev || h->n < 1) return EDGPU_ERR_ARG;
  if (j0 < 0 || j1 > K_cap || j0 > j1) return EDGPU_ERR_ARG;
  if (j0 == 0 && !v0) return EDGPU_ERR_ARG;
  if (workspace_bytes < edgpu_lanczos_reorth_workspace(h->n, K_cap)) return EDGPU_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  if (j0 == j1) return EDGPU_OK;
  const int64_t n = h->n;
  double2* V = reinterpret_cast<double2*>(Vd);
  double2* w = reinterpret_cast<double2*>(wd);
  const unsigned nrb = grid_1d(n, 256);
  unsigned char* ws = reinterpret_cast<unsigned char*>(workspace);
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    unsigned char* p = ws + off;
    off += (bytes + 255) & ~(size_t)255;
    return p;
  };
  double* pa = reinterpret_cast<double*>(carve(sizeof(double) * nrb));
  double* pn = reinterpret_cast<double*>(carve(sizeof(double) * nrb));
  double2* pd = reinterpret_cast<double2*>(carve(sizeof(double2) * (size_t)(K_cap + 1) * nrb));
  double2* hc = reinterpret_cast<double2*>(carve(sizeof(double2) * (size_t)(K_cap + 1)));
  double* pnp = reinterpret_cast<double*>(carve(sizeof(double) * (size_t)((n + 31) / 32 + 1)));
  double* coop = reinterpret_cast<double*>(carve(reorth_coop_scratch_bytes()));
  if (off > workspace_bytes) return EDGPU_ERR_WORKSPACE;
  if (g_reorth_fused.load()) {
    const int rcc = lanczos_reorth_coop(h, v0, j0, j1, K_cap, Vd, wd, alpha, beta, status_dev, coop, hc, s);
    if (rcc >= 0) return rcc;
  }
  if (j0 == 0) {
    copy_c128_kernel<<<grid_1d(n, 256), 256, 0, s>>>(reinterpret_cast<const double2*>(v0), V, n);
    note_launch();
  }
  int rc = check_launch();
  if (rc) return rc;
  for (int j = j0; j < j1; ++j) {
    const double2* vj = V + (int64_t)j * n;
    // w = H v_j ; alpha partials
    dim3 grid(nrb, 1), block(1, 256);
    if (h->val_c)
      spmm_alpha_kernel<double, true><<<grid, block, sizeof(double) * 256, s>>>(n, h->row_ptr, h->col, h->val_c, 1,
                                                                                vj, w, pa, 1);
    else
      spmm_alpha_kernel<double, false><<<grid, block, sizeof(double) * 256, s>>>(n, h->row_ptr, h->col, h->val_r, 1,
                                                                                 vj, w, pa, 1); note_launch();
    reorth_alpha_update_kernel<<<nrb, 256, 0, s>>>(n, w, vj, j > 0 ? V + (int64_t)(j - 1) * n : nullptr, pa, nrb,
                                                   alpha, beta, j, pn); note_launch();
    if ((rc = check_launch())) return rc;
    if (j + 1 >= K_cap) break;
    // two passes of classical Gram-Schmidt against V[0..j]; the second pass also forms the
    // per-block partial norms of the final w
    const int m = j + 1;
    const unsigned prb = (unsigned)((n + 31) / 32);
    for (int pass = 0; pass < 2; ++pass) {
      dot_per_k_kernel<<<m, 256, 0, s>>>(V, m, n, w, hc); note_launch();
      project_out_kernel<<<prb, 256, 0, s>>>(V, m, n, hc, w, pnp, pass == 1); note_launch();
    }
    reorth_normalize_kernel<<<nrb, 256, 0, s>>>(n, w, V + (int64_t)(j + 1) * n, pnp, (int)prb, beta, j, status_dev); note_launch();
    (void)pd;
    (void)pn;
    if ((rc = check_launch())) return rc;
  }
  return EDGPU_OK;
}

extern "C" int edgpu_combine(const double* V, int K, int64_t n, const double* C, int M, double* X, void* stream) {
  if (!V || !C || !X || K < 1 || M < 1 || n < 1) return EDGPU_ERR_ARG;
  dim3 grid(grid_1d(n, 256) > 64 ? 64 : grid_1d(n, 256), M);
  combine_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const double2*>(V), K, n,
                                                        reinterpret_cast<const double2*>(C), M,
                                                        reinterpret_cast<double2*>(X)); note_launch();
  return check_launch();
}

extern "C" size_t edgpu_cfrac_f32_workspace(int K, int R) { return 2 * sizeof(float) * (size_t)K * R + 512; }

extern "C" int edgpu_cfrac_f32(const double* alpha, const double* beta, const int32_t* k_len, int K, int R,
                               const double* omega, int n_omega, double delta, const double* e, const double* scale,
                               double* g, void* workspace, size_t workspace_bytes, void* stream) {
  if (!alpha || !beta || !k_len || !omega || !e || !g || K < 1 || R < 0 || n_omega < 0) return EDGPU_ERR_ARG;
  const int64_t tot = (int64_t)R * n_omega;
  if (tot == 0) return EDGPU_OK;
  if (!workspace || workspace_bytes < edgpu_cfrac_f32_workspace(K, R)) return EDGPU_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  float* ap = reinterpret_cast<float*>(workspace);
  float* b2 = ap + (size_t)K * R;
  const int64_t tk = (int64_t)K * R;
  cfrac_prep_kernel<<<(unsigned)((tk + 255) / 256), 256, 0, s>>>(alpha, beta, k_len, K, R, e, ap, b2);
  note_launch();
  cfrac_f32_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(ap, b2, k_len, K, R, omega, n_omega, delta, scale,
                                                               reinterpret_cast<double2*>(g));
  note_launch();
  return check_launch();
}

extern "C" int edgpu_cfrac(const double* alpha, const double* beta, const int32_t* k_len, int K, int R,
                           const double* omega, int n_omega, double delta, const double* e, const double* scale,
                           double* g, void* stream) {
  if (!alpha || !beta || !k_len || !omega || !e || !g || K < 1 || R < 0 || n_omega < 0) return EDGPU_ERR_ARG;
  const int64_t tot = (int64_t)R * n_omega;
  if (tot == 0) return EDGPU_OK;
  const int threads = 256;
  cfrac_kernel<<<(unsigned)((tot + threads - 1) / threads), threads, 0, (cudaStream_t)stream>>>(
      alpha, beta, k_len, K, R, omega, n_omega, delta, e, scale, reinterpret_cast<double2*>(g)); note_launch();
  return check_launch();
}

// =======================================================================================
// Small sectors: one CTA per run, the whole Krylov loop in one persistent launch.
// =======================================================================================
namespace edgpu {

constexpr int kSmallThreads = 512;
constexpr int kSmallBatch = 8;  // CSR entries loaded together per row

// Deterministic block sum (fixed thread -> partial mapping and fixed tree).
__device__ __forceinline__ double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    double t = lane < nw ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) red[32] = t;
  }
  __syncthreads();
  return red[32];
}

__device__ __forceinline__ double2 to_v(double2 a, double) { return a; }
__device__ __forceinline__ float2 to_v(double2 a, float) { return make_float2((float)a.x, (float)a.y); }

// Upstream's Lanczos recurrence (finite.py:1974-1992) for run r entirely in shared memory:
// x = v_j, p = v_{j-1}, y = H v_j then w.  One CTA per run, persistent over runs.
template <typename T, bool VALC>
__global__ void __launch_bounds__(kSmallThreads) lanczos_small_kernel(
    int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ col, const T* __restrict__ vals, int R,
    const double2* __restrict__ v0, const int32_t* __restrict__ k_max, int K, double* __restrict__ alpha,
    double* __restrict__ beta, int32_t* status) {
  using V = typename Cx<T>::V;
  extern __shared__ __align__(16) unsigned char sm[];
  V* A = reinterpret_cast<V*>(sm);
  V* B = A + n;
  V* Cv = B + n;
  double* red = reinterpret_cast<double*>(Cv + n);
  const int tid = threadIdx.x, bs = blockDim.x;
  for (int r = blockIdx.x; r < R; r += gridDim.x) {
    const int km = k_max[r];
    if (km <= 0) continue;
    for (int64_t i = tid; i < n; i += bs) {
      A[i] = to_v(v0[i * R + r], T(0));
      B[i] = to_v(make_double2(0.0, 0.0), T(0));
    }
    __syncthreads();
    V* x = A;
    V* p = B;
    V* y = Cv;
    double bprev = 0.0;
    for (int j = 0; j < km; ++j) {
      double acc = 0.0;
      for (int64_t i = tid; i < n; i += bs) {
        T yr = 0, yi = 0;
        const int64_t e1 = rp[i + 1];
        for (int64_t e = rp[i]; e < e1; ++e) {
          const V xv = x[col[e]];
          if (VALC) {
            const T hr = vals[2 * e], hi = vals[2 * e + 1];
            yr += hr * xv.x - hi * xv.y;
            yi += hr * xv.y + hi * xv.x;
          } else {
            const T h = vals[e];
            yr += h * xv.x;
            yi += h * xv.y;
          }
        }
        V yv;
        yv.x = yr;
        yv.y = yi;
        y[i] = yv;
        const V xi = x[i];
        acc += (double)yr * (double)xi.x + (double)yi * (double)xi.y;
      }
      const double a = block_sum(acc, red);
      if (tid == 0) alpha[(int64_t)r * K + j] = a;
      if (j + 1 == km) break;
      acc = 0.0;
      const T af = (T)a, bf = (T)bprev;
      for (int64_t i = tid; i < n; i += bs) {
        V w = y[i];
        const V xi = x[i];
        const V pi = p[i];
        w.x = (w.x - af * xi.x) - bf * pi.x;
        w.y = (w.y - af * xi.y) - bf * pi.y;
        y[i] = w;
        acc += (double)w.x * (double)w.x + (double)w.y * (double)w.y;
      }
      const double b = sqrt(block_sum(acc, red));
      if (tid == 0) {
        beta[(int64_t)r * K + j] = b;
        if (!(b > 0.0)) atomicExch(status, (int32_t)(b == 0.0 ? EDGPU_ERR_BREAKDOWN : EDGPU_ERR_NAN));
      }
      const T inv = b > 0.0 ? (T)(1.0 / b) : (T)0;
      for (int64_t i = tid; i < n; i += bs) {
        const V w = y[i];
        V o;
        o.x = w.x * inv;
        o.y = w.y * inv;
        p[i] = o;  // overwrite v_{j-1} with v_{j+1}
      }
      __syncthreads();
      V* t = p;
      p = x;
      x = t;
      bprev = b;
    }
    __syncthreads();
  }
}

// The double-float recurrence with one shared-memory vector per run.  The H v_j pass
// gathers x = v_j from anywhere in the sector, but every other access to a vector touches
// only the thread's own rows (i = tid, tid + THREADS, ...), so v_{j-1} lives in a per-CTA
// slice of global memory (the Lanczos workspace; each element is read and written only by
// the thread that owns its row, so no fence is needed) and only x occupies shared memory.
// Pass 1 overwrites p = v_{j-1} with H v_j - beta_{j-1} v_{j-1} while summing
// alpha_j = v_j . H v_j from the same row values; pass 2, after the SpMV of every thread
// has finished (the alpha sum's barriers), forms w = p - alpha_j v_j, moves v_j into p and
// w into x; pass 3 normalises x in place.  (The subtractions run in the order
// (H v - beta p) - alpha v instead of upstream's (H v - alpha v) - beta p, a difference at
// the 2^-48 rounding level.)  At 16 + 4 bytes per row of shared memory (vector and cached
// row pointers) five or six CTAs fit on an SM, so a batch of runs the size of a RIXS map
// (hundreds of runs) runs as one wave.  Every thread forms beta and 1/beta itself from the
// broadcast sum (double-float square root and reciprocal, a few FP32 instructions), so no
// barrier publishes them; the last thread converts alpha and beta to FP64 for the outputs.
template <int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) lanczos_small_df_kernel(
    int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ col, const float2* __restrict__ hv, int R,
    const double2* __restrict__ v0, const int32_t* __restrict__ k_max, int K, double* __restrict__ alpha,
    double* __restrict__ beta, int32_t* status, float4* __restrict__ pbuf) {
  // vectors as float4 (re.hi, im.hi, re.lo, im.lo): .xy and .zw are the packed high and
  // low parts that the float2 instructions take directly
  extern __shared__ __align__(16) unsigned char sm[];
  float4* x = reinterpret_cast<float4*>(sm);
  dfl* red = reinterpret_cast<dfl*>(x + n);                // two reduction buffers
  int32_t* srp = reinterpret_cast<int32_t*>(red + kDfRed);  // row pointers, cached once
  float4* __restrict__ p = pbuf + (size_t)blockIdx.x * (size_t)n;
  constexpr int NW = THREADS / 32;
  const int tid = threadIdx.x;
  const dfl zero = {0.f, 0.f};
  for (int64_t i = tid; i <= n; i += THREADS) srp[i] = (int32_t)rp[i];
  for (int r = blockIdx.x; r < R; r += gridDim.x) {
    const int km = k_max[r];
    if (km <= 0) continue;
    for (int64_t i = tid; i < n; i += THREADS) {
      const double2 v = v0[i * R + r];
      const dfl re = df_split(v.x), im = df_split(v.y);
      x[i] = make_float4(re.hi, im.hi, re.lo, im.lo);
      p[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    dfl bprev = zero;
    for (int j = 0; j < km; ++j) {
      const dfl nb = {-bprev.hi, -bprev.lo};
      dacc2 acc = {{0.f, 0.f}, {0.f, 0.f}};
      for (int64_t i = tid; i < n; i += THREADS) {
        const float4 pi = p[i];  // issued before the row's products, used after them
        dacc2 y = {{0.f, 0.f}, {0.f, 0.f}};
        const int e1 = srp[i + 1];
        for (int e = srp[i]; e < e1; e += kSmallBatch) {
          int c[kSmallBatch];
          float2 hh[kSmallBatch];
#pragma unroll
          for (int u = 0; u < kSmallBatch; ++u) {
            const bool ok = e + u < e1;
            c[u] = ok ? __ldg(col + e + u) : 0;
            hh[u] = ok ? __ldg(hv + e + u) : make_float2(0.f, 0.f);
          }
#pragma unroll
          for (int u = 0; u < kSmallBatch; ++u) {
            if (e + u < e1) {
              const float4 xv = x[c[u]];
              dacc2_fma(y, {hh[u].x, hh[u].y}, make_float2(xv.x, xv.y), make_float2(xv.z, xv.w));
            }
          }
        }
        const dfl2 h = dacc2_val(y);
        const float4 xi = x[i];
        dacc2_fma2(acc, h, make_float2(xi.x, xi.y), make_float2(xi.z, xi.w));
        const dfl2 w = df2_fma_s(h, {make_float2(pi.x, pi.y), make_float2(pi.z, pi.w)}, nb);
        p[i] = make_float4(w.hi.x, w.hi.y, w.lo.x, w.lo.y);
      }
      const dfl a = df_block_sum2<NW>(dacc2_total(acc), red);
      if (tid == THREADS - 1) alpha[(int64_t)r * K + j] = df_val(a);
      if (j + 1 == km) break;
      const dfl na = {-a.hi, -a.lo};
      acc = {{0.f, 0.f}, {0.f, 0.f}};
      for (int64_t i = tid; i < n; i += THREADS) {
        const float4 wv = p[i], xi = x[i];
        const dfl2 w = df2_fma_s({make_float2(wv.x, wv.y), make_float2(wv.z, wv.w)},
                                 {make_float2(xi.x, xi.y), make_float2(xi.z, xi.w)}, na);
        p[i] = xi;  // v_j: the next step's v_{j-1}
        x[i] = make_float4(w.hi.x, w.hi.y, w.lo.x, w.lo.y);
        dacc2_fma2(acc, w, w.hi, w.lo);
      }
      bprev = df_sqrt(df_block_sum2<NW>(dacc2_total(acc), red + 40));
      const dfl ib = bprev.hi > 0.f ? df_rcp(bprev) : zero;
      if (tid == THREADS - 1) {
        const double b = df_val(bprev);
        beta[(int64_t)r * K + j] = b;
        if (!(b > 0.0)) atomicExch(status, (int32_t)(b == 0.0 ? EDGPU_ERR_BREAKDOWN : EDGPU_ERR_NAN));
      }
      for (int64_t i = tid; i < n; i += THREADS) {
        const float4 wv = x[i];
        const dfl2 v = df2_mul_s({make_float2(wv.x, wv.y), make_float2(wv.z, wv.w)}, ib);
        x[i] = make_float4(v.hi.x, v.hi.y, v.lo.x, v.lo.y);
      }
      __syncthreads();
    }
    __syncthreads();
  }
}

// Sliced layout of a CSR matrix for the one-CTA-per-run double-float Lanczos.  Rows are
// ordered by length, longest first (a stable counting sort, so equal lengths keep their
// order), and cut into slices of 32 consecutive slots, one slice per warp iteration; slice q
// stores entry e of its lane-th row at soff[q] + 32 e + lane, padded to the slice's longest
// row, so that a warp's loads of the e-th entries of its 32 rows are one contiguous 128-byte
// (columns) and 256-byte (values) line, and the rows of a warp have nearly equal lengths.
// sinfo[slot] = row | (length << 16), or -1 for the padding slots after the last row; the
// stored columns are slots too (the slot that holds the column's row), so the Lanczos kernel
// keeps its vector in slot order and touches a warp's own rows contiguously.
// Built by one CTA: the counting sort's histogram with atomics (order-free), the stable
// placement by warp 0 with __match_any_sync ranks, then the fill by every thread.  When the
// slices would need more than `cap` entries (possible only for rows with repeated columns)
// every slot gets length 0 and *status EDGPU_ERR_WORKSPACE, so nothing reads past the arrays.
__global__ void __launch_bounds__(1024) df_slices_kernel(int64_t n, const int64_t* __restrict__ rp,
                                                         const int32_t* __restrict__ col,
                                                         const float2* __restrict__ hv, int32_t* __restrict__ sinfo,
                                                         int32_t* __restrict__ soff, int32_t* __restrict__ ecol,
                                                         float2* __restrict__ eval, int64_t cap, int32_t* status) {
  extern __shared__ int32_t hist[];  // [n + 1] bucket offsets (row lengths 0..n)
  __shared__ int32_t s_max;
  __shared__ int32_t s_over;
  const int tid = threadIdx.x;
  const int npad = (int)((n + 31) & ~(int64_t)31), nslices = npad >> 5;
  if (tid == 0) {
    s_max = 0;
    s_over = 0;
  }
  __syncthreads();
  int lmax = 0;
  for (int64_t i = tid; i < n; i += blockDim.x) lmax = max(lmax, (int)(rp[i + 1] - rp[i]));
  atomicMax(&s_max, lmax);
  __syncthreads();
  if (s_max > n) {  // repeated columns: no sliced layout
    for (int q = tid; q < npad; q += blockDim.x) sinfo[q] = q < n ? q : -1;
    for (int q = tid; q <= nslices; q += blockDim.x) soff[q] = 0;
    if (tid == 0) atomicExch(status, (int32_t)EDGPU_ERR_WORKSPACE);
    return;
  }
  const int L = s_max;
  for (int k = tid; k <= L; k += blockDim.x) hist[k] = 0;
  __syncthreads();
  for (int64_t i = tid; i < n; i += blockDim.x) atomicAdd(&hist[L - (int)(rp[i + 1] - rp[i])], 1);
  __syncthreads();
  if (tid == 0) {
    int run = 0;
    for (int k = 0; k <= L; ++k) {
      const int c = hist[k];
      hist[k] = run;
      run += c;
    }
  }
  __syncthreads();
  if (tid < 32) {
    const unsigned lt = (1u << tid) - 1u;
    for (int64_t c0 = 0; c0 < n; c0 += 32) {
      const int64_t i = c0 + tid;
      const int len = i < n ? (int)(rp[i + 1] - rp[i]) : 0;
      const int key = i < n ? L - len : -1;
      const unsigned same = __match_any_sync(0xffffffffu, key);
      const int base = key >= 0 ? hist[key] : 0;
      if (i < n) sinfo[base + __popc(same & lt)] = (int32_t)i | (len << 16);
      __syncwarp();
      if (key >= 0 && (__ffs(same) - 1) == tid) hist[key] = base + __popc(same);
      __syncwarp();
    }
  }
  for (int q = (int)n + tid; q < npad; q += blockDim.x) sinfo[q] = -1;
  __syncthreads();
  // the bucket offsets are spent: hist becomes the slot of each row
  for (int q = tid; q < (int)n; q += blockDim.x) hist[sinfo[q] & 0xffff] = q;
  __syncthreads();
  if (tid == 0) {
    int64_t off = 0;
    soff[0] = 0;
    for (int q = 0; q < nslices; ++q) {
      off += 32 * (int64_t)(sinfo[32 * q] >> 16);  // the slice's first row is its longest
      soff[q + 1] = (int32_t)off;
    }
    if (off > cap) s_over = 1;
  }
  __syncthreads();
  if (s_over) {
    for (int q = tid; q < npad; q += blockDim.x) sinfo[q] = sinfo[q] < 0 ? -1 : (sinfo[q] & 0xffff);
    for (int q = tid; q <= nslices; q += blockDim.x) soff[q] = 0;
    if (tid == 0) atomicExch(status, (int32_t)EDGPU_ERR_WORKSPACE);
    return;
  }
  for (int q = tid; q < npad; q += blockDim.x) {
    const int info = sinfo[q];
    const int sl = q >> 5;
    const int m = (soff[sl + 1] - soff[sl]) >> 5;
    const int64_t base = soff[sl] + (q & 31);
    const int len = info < 0 ? 0 : (info >> 16);
    const int64_t e0 = info < 0 ? 0 : rp[info & 0xffff];
    for (int e = 0; e < m; ++e) {
      ecol[base + 32 * e] = e < len ? hist[col[e0 + e]] : 0;
      eval[base + 32 * e] = e < len ? hv[e0 + e] : make_float2(0.f, 0.f);
    }
  }
}

// Entries the sliced layout can need: every slice but the first is no wider than the
// shortest row of the slice before it, so the padding beyond nnz is at most 32 times the
// longest row, itself at most n for rows without repeated columns.
static int64_t df_slices_cap(int64_t n, int64_t nnz) { return nnz + 32 * n; }

// lanczos_small_df_kernel on the sliced layout: thread tid walks the slots tid, tid +
// THREADS, ... (a warp takes whole slices), so its rows and their order follow the slots;
// both vectors are kept in slot order (the stored columns are slots), so every access but
// the H v gathers is contiguous.  The arithmetic of every row and vector element is that of
// lanczos_small_df_kernel; only the rows' assignment to threads, and so the order of the
// per-thread partial sums of alpha and beta, differ.
template <int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) lanczos_sliced_df_kernel(
    int64_t n, const int32_t* __restrict__ g_sinfo, const int32_t* __restrict__ g_soff,
    const int32_t* __restrict__ ecol, const float2* __restrict__ eval, int R, const double2* __restrict__ v0,
    const int32_t* __restrict__ k_max, int K, double* __restrict__ alpha, double* __restrict__ beta, int32_t* status,
    float4* __restrict__ pbuf) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int npad = (int)((n + 31) & ~(int64_t)31), nslices = npad >> 5;
  float4* x = reinterpret_cast<float4*>(sm);  // in slot order, zero in the padding slots
  dfl* red = reinterpret_cast<dfl*>(x + npad);
  int32_t* sinfo = reinterpret_cast<int32_t*>(red + kDfRed);
  int32_t* soff = sinfo + npad;
  float4* __restrict__ p = pbuf + (size_t)blockIdx.x * (size_t)npad;
  constexpr int NW = THREADS / 32;
  const int tid = threadIdx.x;
  const dfl zero = {0.f, 0.f};
  for (int q = tid; q < npad; q += THREADS) sinfo[q] = g_sinfo[q];
  for (int q = tid; q <= nslices; q += THREADS) soff[q] = g_soff[q];
  for (int r = blockIdx.x; r < R; r += gridDim.x) {
    const int km = k_max[r];
    if (km <= 0) continue;
    for (int q = tid; q < npad; q += THREADS) {
      const int info = sinfo[q];
      float4 xv = make_float4(0.f, 0.f, 0.f, 0.f);
      if (info >= 0) {
        const double2 v = v0[(int64_t)(info & 0xffff) * R + r];
        const dfl re = df_split(v.x), im = df_split(v.y);
        xv = make_float4(re.hi, im.hi, re.lo, im.lo);
      }
      x[q] = xv;
      p[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    dfl bprev = zero;
    for (int j = 0; j < km; ++j) {
      const dfl nb = {-bprev.hi, -bprev.lo};
      dacc2 acc = {{0.f, 0.f}, {0.f, 0.f}};
      for (int q = tid; q < npad; q += THREADS) {
        const int info = sinfo[q];
        if (info < 0) continue;
        const float4 pq = p[q];
        const int len = info >> 16;
        const int64_t base = soff[q >> 5] + (q & 31);
        dacc2 y = {{0.f, 0.f}, {0.f, 0.f}};
        for (int e = 0; e < len; e += kSmallBatch) {
          int c[kSmallBatch];
          float2 hh[kSmallBatch];
#pragma unroll
          for (int u = 0; u < kSmallBatch; ++u) {
            const bool ok = e + u < len;
            c[u] = ok ? __ldg(ecol + base + 32 * (e + u)) : 0;
            hh[u] = ok ? __ldg(eval + base + 32 * (e + u)) : make_float2(0.f, 0.f);
          }
#pragma unroll
          for (int u = 0; u < kSmallBatch; ++u) {
            if (e + u < len) {
              const float4 xv = x[c[u]];
              dacc2_fma(y, {hh[u].x, hh[u].y}, make_float2(xv.x, xv.y), make_float2(xv.z, xv.w));
            }
          }
        }
        const dfl2 h = dacc2_val(y);
        const float4 xi = x[q];
        dacc2_fma2(acc, h, make_float2(xi.x, xi.y), make_float2(xi.z, xi.w));
        const dfl2 w = df2_fma_s(h, {make_float2(pq.x, pq.y), make_float2(pq.z, pq.w)}, nb);
        p[q] = make_float4(w.hi.x, w.hi.y, w.lo.x, w.lo.y);
      }
      const dfl a = df_block_sum2<NW>(dacc2_total(acc), red);
      if (tid == THREADS - 1) alpha[(int64_t)r * K + j] = df_val(a);
      if (j + 1 == km) break;
      const dfl na = {-a.hi, -a.lo};
      acc = {{0.f, 0.f}, {0.f, 0.f}};
      for (int q = tid; q < npad; q += THREADS) {
        if (sinfo[q] < 0) continue;
        const float4 wv = p[q], xi = x[q];
        const dfl2 w = df2_fma_s({make_float2(wv.x, wv.y), make_float2(wv.z, wv.w)},
                                 {make_float2(xi.x, xi.y), make_float2(xi.z, xi.w)}, na);
        p[q] = xi;  // v_j: the next step's v_{j-1}
        x[q] = make_float4(w.hi.x, w.hi.y, w.lo.x, w.lo.y);
        dacc2_fma2(acc, w, w.hi, w.lo);
      }
      bprev = df_sqrt(df_block_sum2<NW>(dacc2_total(acc), red + 40));
      const dfl ib = bprev.hi > 0.f ? df_rcp(bprev) : zero;
      if (tid == THREADS - 1) {
        const double b = df_val(bprev);
        beta[(int64_t)r * K + j] = b;
        if (!(b > 0.0)) atomicExch(status, (int32_t)(b == 0.0 ? EDGPU_ERR_BREAKDOWN : EDGPU_ERR_NAN));
      }
      for (int q = tid; q < npad; q += THREADS) {  // the padding slots stay zero
        const float4 wv = x[q];
        const dfl2 v = df2_mul_s({make_float2(wv.x, wv.y), make_float2(wv.z, wv.w)}, ib);
        x[q] = make_float4(v.hi.x, v.hi.y, v.lo.x, v.lo.y);
      }
      __syncthreads();
    }
    __syncthreads();
  }
}

static size_t sliced_df_smem_bytes(int64_t n) {
  const int64_t npad = (n + 31) & ~(int64_t)31;
  return sizeof(float4) * (size_t)npad + kDfRed * sizeof(dfl) + sizeof(int32_t) * (size_t)(npad + npad / 32 + 1) + 16;
}

// Shared memory that decides whether a sector takes the one-CTA-per-run path (unchanged by
// the one-vector form of the double-float kernel, so that the same sectors take it).
size_t small_smem_bytes(int64_t n, int precision) {
  if (precision == 3)
    return 2 * sizeof(float4) * (size_t)n + kDfRed * sizeof(dfl) + sizeof(int32_t) * (size_t)(n + 1) + 16;
  const size_t v = precision == 1 ? sizeof(float2) : sizeof(double2);
  return 3 * v * (size_t)n + 68 * sizeof(double) + 16;
}

// Shared memory of one lanczos_small_df_kernel CTA: x, the reduction buffers, row pointers.
static size_t small_df_smem_bytes(int64_t n) {
  return sizeof(float4) * (size_t)n + kDfRed * sizeof(dfl) + sizeof(int32_t) * (size_t)(n + 1) + 16;
}

bool small_fits(int64_t n, int precision) { return small_smem_bytes(n, precision) <= 200 * 1024; }

template <typename T, bool VALC>
int launch_small(const edgpu_csr* h, const T* vals, const double* v0, int R, const int32_t* k_max, int K,
                 double* alpha, double* beta, int32_t* status, int precision, cudaStream_t s) {
  const size_t smem = small_smem_bytes(h->n, precision);
  auto kern = lanczos_small_kernel<T, VALC>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSmallThreads, smem);
  if (per_sm < 1) per_sm = 1;
  int grid = grid_cap() * per_sm;
  if (grid > R) grid = R;
  kern<<<grid, kSmallThreads, smem, s>>>(h->n, h->row_ptr, h->col, vals, R, reinterpret_cast<const double2*>(v0), k_max,
                                         K, alpha, beta, status);
  note_launch();
  return check_launch();
}

// CTA slots per SM that the one-CTA-per-run double-float Lanczos leaves free (process-wide,
// default 0), so that kernels of a pipeline running concurrently on another stream find room
// on every SM instead of waiting for the persistent grid to drain.
static std::atomic<int> g_small_reserve{0};
extern "C" void edgpu_set_small_reserve(int slots) { g_small_reserve.store(slots > 0 ? slots : 0); }

// CTA size: the largest of 512, 256, 192, 160 and 128 threads (64 registers a thread at the
// occupancy each is compiled for) whose CTAs cover the R runs in the fewest waves with one
// slot per SM kept back.  It depends only on (n, R) and the GPU, never on the reserve, so a
// run's reduction order, and its result bits, do not change with concurrent work; the
// reserve only limits how many of the CTAs are resident at once.  On the 1770-row RIXS
// final-state sector with 750 runs this is 160 threads, five CTAs per SM, one wave.
// The sliced layout is used when the smallest workspace edgpu_lanczos accepts for (n, R, K)
// holds it next to the per-CTA vectors (a function of the problem only, so a given problem
// always takes the same path); otherwise the kernel reads the CSR arrays directly.
using SmallDfKern = void (*)(int64_t, const int64_t*, const int32_t*, const float2*, int, const double2*,
                             const int32_t*, int, double*, double*, int32_t*, float4*);
using SlicedDfKern = void (*)(int64_t, const int32_t*, const int32_t*, const int32_t*, const float2*, int,
                              const double2*, const int32_t*, int, double*, double*, int32_t*, float4*);
static const int kDfThreads[5] = {512, 256, 192, 160, 128};

// Process-wide CTA-size choice for the double-float one-CTA-per-run Lanczos (index into
// kDfThreads, or -1 for the rule below); set by the engine's autotuner around a call.
static std::atomic<int> g_df_cta{-1};
extern "C" void edgpu_set_lanczos_cta(int index) { g_df_cta.store(index >= 0 && index < 5 ? index : -1); }

static int pick_df_config(const void* const* kerns, size_t smem, int R, int* per_sm_out) {
  const int nsm = grid_cap();
  const int forced = g_df_cta.load();
  if (forced >= 0) {
    cudaFuncSetAttribute(kerns[forced], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kerns[forced], kDfThreads[forced], smem);
    if (per_sm >= 1) {
      *per_sm_out = per_sm;
      return forced;
    }
    cudaGetLastError();
  }
  int best = -1, best_waves = 0;
  for (int c = 0; c < 5; ++c) {
    cudaFuncSetAttribute(kerns[c], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kerns[c], kDfThreads[c], smem);
    if (per_sm < 1) continue;
    const int64_t slots = (int64_t)nsm * (per_sm > 1 ? per_sm - 1 : 1);
    const int waves = (int)((R + slots - 1) / slots);
    if (best < 0 || waves < best_waves) {
      best = c;
      best_waves = waves;
      *per_sm_out = per_sm;
    }
  }
  return best;
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

int launch_small_df(const edgpu_csr* h, const double* v0, int R, const int32_t* k_max, int K, double* alpha,
                    double* beta, int32_t* status, void* ws, cudaStream_t s) {
  static const SmallDfKern csr_kerns[5] = {lanczos_small_df_kernel<512, 2>, lanczos_small_df_kernel<256, 4>,
                                           lanczos_small_df_kernel<192, 5>, lanczos_small_df_kernel<160, 6>,
                                           lanczos_small_df_kernel<128, 8>};
  static const SlicedDfKern sl_kerns[5] = {lanczos_sliced_df_kernel<512, 2>, lanczos_sliced_df_kernel<256, 4>,
                                           lanczos_sliced_df_kernel<192, 5>, lanczos_sliced_df_kernel<160, 6>,
                                           lanczos_sliced_df_kernel<128, 8>};
  const int64_t n = h->n, nnz = h->nnz;
  const int64_t npad = (n + 31) & ~(int64_t)31, nslices = npad / 32;
  const int nsm = grid_cap();
  const int reserve = g_small_reserve.load();
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~(uintptr_t)255);
  // sliced layout: per-CTA vectors, slot table, slice offsets, columns, values
  if (n <= 32767) {
    const size_t smem = sliced_df_smem_bytes(n);
    int per_sm = 1;
    const int c = pick_df_config(reinterpret_cast<const void* const*>(sl_kerns), smem, R, &per_sm);
    if (c >= 0) {
      int grid = nsm * (per_sm - reserve > 0 ? per_sm - reserve : 1);
      if (grid > R) grid = R;
      const int64_t cap = df_slices_cap(n, nnz);
      const size_t b_p = align256(sizeof(float4) * (size_t)npad * (size_t)(R < nsm * per_sm ? R : nsm * per_sm));
      const size_t b_info = align256(sizeof(int32_t) * (size_t)npad);
      const size_t b_off = align256(sizeof(int32_t) * (size_t)(nslices + 1));
      const size_t b_col = align256(sizeof(int32_t) * (size_t)cap);
      const size_t b_val = align256(sizeof(float2) * (size_t)cap);
      if (256 + b_p + b_info + b_off + b_col + b_val <= edgpu_lanczos_workspace(n, R, K, 3)) {
        float4* pbuf = reinterpret_cast<float4*>(base);
        int32_t* sinfo = reinterpret_cast<int32_t*>(base + b_p);
        int32_t* soff = reinterpret_cast<int32_t*>(base + b_p + b_info);
        int32_t* ecol = reinterpret_cast<int32_t*>(base + b_p + b_info + b_off);
        float2* eval = reinterpret_cast<float2*>(base + b_p + b_info + b_off + b_col);
        const size_t hist_bytes = sizeof(int32_t) * (size_t)(n + 1);
        cudaFuncSetAttribute(df_slices_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hist_bytes);
        df_slices_kernel<<<1, 1024, hist_bytes, s>>>(n, h->row_ptr, h->col, reinterpret_cast<const float2*>(h->val_df),
                                                     sinfo, soff, ecol, eval, cap, status);
        note_launch();
        sl_kerns[c]<<<grid, kDfThreads[c], smem, s>>>(n, sinfo, soff, ecol, eval, R,
                                                       reinterpret_cast<const double2*>(v0), k_max, K, alpha, beta,
                                                       status, pbuf);
        note_launch();
        return check_launch();
      }
    }
  }
  const size_t smem = small_df_smem_bytes(n);
  int per_sm = 1;
  const int c = pick_df_config(reinterpret_cast<const void* const*>(csr_kerns), smem, R, &per_sm);
  if (c < 0) return EDGPU_ERR_ARG;
  int grid = nsm * (per_sm - reserve > 0 ? per_sm - reserve : 1);
  if (grid > R) grid = R;
  csr_kerns[c]<<<grid, kDfThreads[c], smem, s>>>(n, h->row_ptr, h->col, reinterpret_cast<const float2*>(h->val_df), R,
                                                 reinterpret_cast<const double2*>(v0), k_max, K, alpha, beta, status,
                                                 reinterpret_cast<float4*>(base));
  note_launch();
  return check_launch();
}

int lanczos_small(const edgpu_csr* h, const double* v0, int R, const int32_t* k_max, int K, int precision,
                  double* alpha, double* beta, int32_t* status, void* ws, cudaStream_t s) {
  if (precision == 3) {
    if (h->val_df && !h->val_c) return launch_small_df(h, v0, R, k_max, K, alpha, beta, status, ws, s);
    precision = 0;  // complex H: FP64
  }
  if (precision == 0) {
    if (h->val_c) return launch_small<double, true>(h, h->val_c, v0, R, k_max, K, alpha, beta, status, 0, s);
    return launch_small<double, false>(h, h->val_r, v0, R, k_max, K, alpha, beta, status, 0, s);
  }
  if (h->val_cf) return launch_small<float, true>(h, h->val_cf, v0, R, k_max, K, alpha, beta, status, 1, s);
  if (!h->val_rf) return EDGPU_ERR_ARG;
  return launch_small<float, false>(h, h->val_rf, v0, R, k_max, K, alpha, beta, status, 1, s);
}

// ---------------------------------------------------------------------------------------
// Shifted solves (z - H) x = y for many z from one Krylov space, CTA per right-hand side.
// The Lanczos vectors v_{j-1}, v_j and w live in shared memory; each v_j is also written to
// V[rhs][j][n] for assembling x(z) = |y| V (z - T)^{-1} e_1 afterwards.  No
// reorthogonalisation: the three-term relation H V = V T + b v e^T holds to rounding even
// after orthogonality is lost, so the residual estimate below stays valid and the loop
// simply runs until it is met.  Thread t < nz tracks shift z_t: LU pivots
// d_k = (z - a_k) - b_{k-1}^2 / d_{k-1} and the last component q_m of (z - T_m)^{-1} e_1,
// so the residual ||r|| / ||y|| = b_{m-1} |q_m| costs O(1) per step.
// Replaces upstream's per-energy BiCGSTAB (spectra.py:962,1080).
// ---------------------------------------------------------------------------------------
template <bool VALC>
__global__ void __launch_bounds__(kSmallThreads) shifted_small_kernel(
    int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ col, const double* __restrict__ vals,
    int n_rhs, const double2* __restrict__ Y, const double2* __restrict__ zs, int nz, int k_cap, double tol,
    double2* __restrict__ V, double* __restrict__ alpha, double* __restrict__ beta, int32_t* __restrict__ m_out,
    double* __restrict__ ynorm_out, int32_t* status) {
  extern __shared__ __align__(16) unsigned char sm[];
  double2* X = reinterpret_cast<double2*>(sm);
  double2* P = X + n;
  double2* Wv = P + n;
  double* red = reinterpret_cast<double*>(Wv + n);
  const int tid = threadIdx.x, bs = blockDim.x;
  for (int r = blockIdx.x; r < n_rhs; r += gridDim.x) {
    double2* Vr = V + (size_t)r * k_cap * n;
    const double2* y = Y + (size_t)r * n;
    double acc = 0.0;
    for (int64_t i = tid; i < n; i += bs) acc += y[i].x * y[i].x + y[i].y * y[i].y;
    const double yn = sqrt(block_sum(acc, red));
    if (tid == 0) ynorm_out[r] = yn;
    if (!(yn > 0.0)) {
      if (tid == 0) m_out[r] = 0;
      continue;
    }
    const double iyn = 1.0 / yn;
    for (int64_t i = tid; i < n; i += bs) {
      const double2 v = make_double2(y[i].x * iyn, y[i].y * iyn);
      X[i] = v;
      P[i] = make_double2(0.0, 0.0);
      Vr[i] = v;
    }
    __syncthreads();
    double2* x = X;
    double2* p = P;
    double2 z = make_double2(0.0, 0.0), d = make_double2(1.0, 0.0), q = make_double2(1.0, 0.0);
    if (tid < nz) z = zs[(size_t)r * nz + tid];
    double bprev = 0.0;
    int m = k_cap;
    for (int j = 0; j < k_cap; ++j) {
      acc = 0.0;
      for (int64_t i = tid; i < n; i += bs) {
        double yr = 0.0, yi = 0.0;
        const int64_t e1 = rp[i + 1];
        for (int64_t e = rp[i]; e < e1; ++e) {
          const double2 xv = x[col[e]];
          if (VALC) {
            const double hr = vals[2 * e], hi = vals[2 * e + 1];
            yr += hr * xv.x - hi * xv.y;
            yi += hr * xv.y + hi * xv.x;
          } else {
            const double h = vals[e];
            yr += h * xv.x;
            yi += h * xv.y;
          }
        }
        Wv[i] = make_double2(yr, yi);
        acc += yr * x[i].x + yi * x[i].y;
      }
      const double a = block_sum(acc, red);
      if (tid == 0) alpha[(size_t)r * k_cap + j] = a;
      acc = 0.0;
      for (int64_t i = tid; i < n; i += bs) {
        double2 t = Wv[i];
        const double2 c = x[i], pv = p[i];
        t.x = (t.x - a * c.x) - bprev * pv.x;
        t.y = (t.y - a * c.y) - bprev * pv.y;
        Wv[i] = t;
        acc += t.x * t.x + t.y * t.y;
      }
      const double b = sqrt(block_sum(acc, red));
      if (tid == 0) beta[(size_t)r * k_cap + j] = b;
      bool ok = true;
      if (tid < nz) {
        double2 dn = make_double2(z.x - a, z.y);
        if (j > 0) {
          const double b2 = bprev * bprev;
          const double den = d.x * d.x + d.y * d.y;
          dn.x -= b2 * d.x / den;
          dn.y += b2 * d.y / den;
        }
        const double2 qn = make_double2(j > 0 ? q.x * bprev : 1.0, j > 0 ? q.y * bprev : 0.0);
        const double den = dn.x * dn.x + dn.y * dn.y;
        q = make_double2((qn.x * dn.x + qn.y * dn.y) / den, (qn.y * dn.x - qn.x * dn.y) / den);
        d = dn;
        ok = b * sqrt(q.x * q.x + q.y * q.y) <= tol;
      }
      const bool conv = __syncthreads_and(ok);
      if (conv || !(b > 0.0) || j + 1 == k_cap) {
        m = j + 1;
        if (tid == 0) {
          if (!(b >= 0.0))
            atomicExch(status, (int32_t)EDGPU_ERR_NAN);
          else if (!conv && b > 0.0)
            atomicExch(status, (int32_t)EDGPU_ERR_NOCONV);
        }
        break;
      }
      const double ib = 1.0 / b;
      double2* vn = Vr + (size_t)(j + 1) * n;
      for (int64_t i = tid; i < n; i += bs) {
        const double2 v = make_double2(Wv[i].x * ib, Wv[i].y * ib);
        p[i] = v;  // v_{j-1} is no longer needed: its buffer becomes v_{j+1}
        vn[i] = v;
      }
      __syncthreads();
      double2* t = p;
      p = x;
      x = t;
      bprev = b;
    }
    if (tid == 0) m_out[r] = m;
    __syncthreads();
  }
}

// The same shifted solves in double-float arithmetic for a real H (values as hi/lo float
// pairs), two vectors per right-hand side as in lanczos_small_df_kernel, each v_j written
// to V[rhs][j] as float4 (re.hi, re.lo, im.hi, im.lo).  The residual estimate only decides
// when to stop, so its LU recurrence runs in FP32 (the pivots keep Im d_k >= Im z > 0, so
// it cannot break down); every thread forms beta and 1/beta from the broadcast sum, and the
// barrier that pools the per-shift verdicts is the only one beyond the two sums.
template <int THREADS>
__global__ void __launch_bounds__(THREADS, 1) shifted_small_df_kernel(
    int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ col, const float2* __restrict__ hv,
    int n_rhs, const double2* __restrict__ Y, const double2* __restrict__ zs, int nz, int k_cap, float tol,
    float4* __restrict__ V, double* __restrict__ alpha, double* __restrict__ beta, int32_t* __restrict__ m_out,
    double* __restrict__ ynorm_out, int32_t* status) {
  extern __shared__ __align__(16) unsigned char sm[];
  float4* A = reinterpret_cast<float4*>(sm);
  float4* B = A + n;
  dfl* red = reinterpret_cast<dfl*>(B + n);
  int32_t* srp = reinterpret_cast<int32_t*>(red + kDfRed);
  constexpr int NW = THREADS / 32;
  const int tid = threadIdx.x;
  const dfl zero = {0.f, 0.f};
  for (int64_t i = tid; i <= n; i += THREADS) srp[i] = (int32_t)rp[i];
  for (int r = blockIdx.x; r < n_rhs; r += gridDim.x) {
    float4* Vr = V + (size_t)r * k_cap * n;
    const double2* y = Y + (size_t)r * n;
    dacc acc = {0.f, 0.f};
    for (int64_t i = tid; i < n; i += THREADS) {
      const double2 v = y[i];
      const dfl re = df_split(v.x), im = df_split(v.y);
      A[i] = make_float4(re.hi, re.lo, im.hi, im.lo);
      dacc_fma(acc, re, re.hi, re.lo);
      dacc_fma(acc, im, im.hi, im.lo);
    }
    const dfl yn = df_sqrt(df_block_sum2<NW>(dacc_val(acc), red));
    if (tid == THREADS - 1) ynorm_out[r] = df_val(yn);
    if (!(yn.hi > 0.f)) {
      if (tid == 0) m_out[r] = 0;
      __syncthreads();
      continue;
    }
    const dfl iyn = df_rcp(yn);
    for (int64_t i = tid; i < n; i += THREADS) {
      const float4 w = A[i];
      const dfl vr = df_mul({w.x, w.y}, iyn), vi = df_mul({w.z, w.w}, iyn);
      const float4 v = make_float4(vr.hi, vr.lo, vi.hi, vi.lo);
      A[i] = v;
      B[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      Vr[i] = v;
    }
    __syncthreads();
    float4* x = A;
    float4* p = B;
    float2 z = make_float2(0.f, 0.f), d = make_float2(1.f, 0.f), q = make_float2(1.f, 0.f);
    if (tid < nz) {
      const double2 zd = zs[(size_t)r * nz + tid];
      z = make_float2((float)zd.x, (float)zd.y);
    }
    dfl bprev = zero;
    int m = k_cap;
    for (int j = 0; j < k_cap; ++j) {
      const dfl nb = {-bprev.hi, -bprev.lo};
      acc = {0.f, 0.f};
      for (int64_t i = tid; i < n; i += THREADS) {
        dacc yr = {0.f, 0.f}, yi = {0.f, 0.f};
        const int e1 = srp[i + 1];
        for (int e = srp[i]; e < e1; e += kSmallBatch) {
          int c[kSmallBatch];
          float2 hh[kSmallBatch];
#pragma unroll
          for (int u = 0; u < kSmallBatch; ++u) {
            const bool ok = e + u < e1;
            c[u] = ok ? __ldg(col + e + u) : 0;
            hh[u] = ok ? __ldg(hv + e + u) : make_float2(0.f, 0.f);
          }
#pragma unroll
          for (int u = 0; u < kSmallBatch; ++u) {
            if (e + u < e1) {
              const dfl h = {hh[u].x, hh[u].y};
              const float4 xv = x[c[u]];
              dacc_fma(yr, h, xv.x, xv.y);
              dacc_fma(yi, h, xv.z, xv.w);
            }
          }
        }
        const dfl hr = dacc_val(yr), hi = dacc_val(yi);
        const float4 xi = x[i], pi = p[i];
        dacc_fma(acc, hr, xi.x, xi.y);
        dacc_fma(acc, hi, xi.z, xi.w);
        const dfl wr = df_fma(hr, nb, {pi.x, pi.y}), wi = df_fma(hi, nb, {pi.z, pi.w});
        p[i] = make_float4(wr.hi, wr.lo, wi.hi, wi.lo);
      }
      const dfl a = df_block_sum2<NW>(dacc_val(acc), red);
      if (tid == THREADS - 1) alpha[(size_t)r * k_cap + j] = df_val(a);
      const dfl na = {-a.hi, -a.lo};
      acc = {0.f, 0.f};
      for (int64_t i = tid; i < n; i += THREADS) {
        const float4 w = p[i], xi = x[i];
        const dfl wr = df_fma({w.x, w.y}, na, {xi.x, xi.y});
        const dfl wi = df_fma({w.z, w.w}, na, {xi.z, xi.w});
        p[i] = make_float4(wr.hi, wr.lo, wi.hi, wi.lo);
        dacc_fma(acc, wr, wr.hi, wr.lo);
        dacc_fma(acc, wi, wi.hi, wi.lo);
      }
      const dfl b = df_sqrt(df_block_sum2<NW>(dacc_val(acc), red + 40));
      if (tid == THREADS - 1) beta[(size_t)r * k_cap + j] = df_val(b);
      bool ok = true;
      if (tid < nz) {
        const float af = a.hi, bp = bprev.hi;
        float2 dn = make_float2(z.x - af, z.y);
        if (j > 0) {
          const float rd = __fdiv_rn(bp * bp, d.x * d.x + d.y * d.y);
          dn.x -= rd * d.x;
          dn.y += rd * d.y;
        }
        const float2 qn = make_float2(j > 0 ? q.x * bp : 1.f, j > 0 ? q.y * bp : 0.f);
        const float rr = __fdiv_rn(1.f, dn.x * dn.x + dn.y * dn.y);
        q = make_float2((qn.x * dn.x + qn.y * dn.y) * rr, (qn.y * dn.x - qn.x * dn.y) * rr);
        d = dn;
        ok = b.hi * sqrtf(q.x * q.x + q.y * q.y) <= tol;
      }
      const bool conv = __syncthreads_and(ok);
      if (conv || !(b.hi > 0.f) || j + 1 == k_cap) {
        m = j + 1;
        if (tid == 0) {
          if (!(b.hi >= 0.f))
            atomicExch(status, (int32_t)EDGPU_ERR_NAN);
          else if (!conv && b.hi > 0.f)
            atomicExch(status, (int32_t)EDGPU_ERR_NOCONV);
        }
        break;
      }
      const dfl ib = df_rcp(b);
      float4* vn = Vr + (size_t)(j + 1) * n;
      for (int64_t i = tid; i < n; i += THREADS) {
        const float4 w = p[i];
        const dfl vr = df_mul({w.x, w.y}, ib), vi = df_mul({w.z, w.w}, ib);
        const float4 v = make_float4(vr.hi, vr.lo, vi.hi, vi.lo);
        p[i] = v;
        vn[i] = v;
      }
      __syncthreads();
      float4* t = p;
      p = x;
      x = t;
      bprev = b;
    }
    if (tid == 0) m_out[r] = m;
    __syncthreads();
  }
}

// coef[r][k][z] = ynorm_r * ((z - T_m)^{-1} e_1)_k by the Thomas algorithm: block per
// right-hand side with its alpha and beta staged in shared memory, thread per shift (one
// FP64 reciprocal per step).  (z - T) has diagonal z - a_k and off-diagonals -b_k; the
// forward-sweep ratios and the solution go through scratch laid out [r][k][z], so a warp's
// accesses are contiguous.  DF writes the coefficients as double-float pairs (float4).
template <bool DF>
__global__ void shifted_coef_kernel(const double* __restrict__ alpha, const double* __restrict__ beta,
                                    const int32_t* __restrict__ m_arr, const double* __restrict__ ynorm,
                                    const double2* __restrict__ zs, int nz, int k_cap, double2* __restrict__ coef,
                                    float4* __restrict__ coef_df, double2* __restrict__ cp,
                                    double2* __restrict__ xs) {
  extern __shared__ double ab[];
  const int r = blockIdx.x;
  const int m = m_arr[r];
  double* a = ab;
  double* b = ab + k_cap;
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    a[k] = alpha[(size_t)r * k_cap + k];
    b[k] = beta[(size_t)r * k_cap + k];
  }
  __syncthreads();
  if (m <= 0) return;
  const double yn = ynorm[r];
  const size_t base = (size_t)r * k_cap * nz;
  for (int zi = threadIdx.x; zi < nz; zi += blockDim.x) {
    const double2 z = zs[(size_t)r * nz + zi];
    double2 cprev = make_double2(0.0, 0.0), dprev = make_double2(0.0, 0.0);
    for (int k = 0; k < m; ++k) {
      double2 den = make_double2(z.x - a[k], z.y);
      double2 rk = make_double2(1.0, 0.0);
      if (k > 0) {
        den.x += b[k - 1] * cprev.x;
        den.y += b[k - 1] * cprev.y;
        rk = make_double2(b[k - 1] * dprev.x, b[k - 1] * dprev.y);
      }
      const double rdd = 1.0 / (den.x * den.x + den.y * den.y);
      const double2 inv = make_double2(den.x * rdd, -den.y * rdd);
      const double bk = (k + 1 < m) ? b[k] : 0.0;
      cprev = make_double2(-bk * inv.x, -bk * inv.y);
      dprev = make_double2(rk.x * inv.x - rk.y * inv.y, rk.x * inv.y + rk.y * inv.x);
      cp[base + (size_t)k * nz + zi] = cprev;
      xs[base + (size_t)k * nz + zi] = dprev;
    }
    double2 xn = dprev;
    for (int k = m - 1; k >= 0; --k) {
      double2 xk = xs[base + (size_t)k * nz + zi];
      if (k + 1 < m) {
        const double2 c = cp[base + (size_t)k * nz + zi];
        xk = make_double2(xk.x - (c.x * xn.x - c.y * xn.y), xk.y - (c.x * xn.y + c.y * xn.x));
      }
      xn = xk;
      const double2 o = make_double2(yn * xk.x, yn * xk.y);
      if (DF) {
        const dfl re = df_split(o.x), im = df_split(o.y);
        coef_df[base + (size_t)k * nz + zi] = make_float4(re.hi, re.lo, im.hi, im.lo);
      } else {
        coef[base + (size_t)k * nz + zi] = o;
      }
    }
  }
}

// X[r][z][i] = sum_k coef[r][k][z] V[r][k][i] (FP64)
__global__ void combine_batched_kernel(const double2* __restrict__ V, const double2* __restrict__ coef,
                                       const int32_t* __restrict__ m_arr, int64_t n, int nz, int k_cap,
                                       double2* __restrict__ X) {
  const int r = blockIdx.z;
  const int zi = blockIdx.y;
  const int m = m_arr[r];
  const double2* c = coef + (size_t)r * k_cap * nz + zi;
  const double2* Vr = V + (size_t)r * k_cap * n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double xr = 0.0, xi = 0.0;
#pragma unroll 8
    for (int k = 0; k < m; ++k) {
      const double2 ck = c[(size_t)k * nz];
      const double2 v = Vr[(size_t)k * n + i];
      xr += ck.x * v.x - ck.y * v.y;
      xi += ck.x * v.y + ck.y * v.x;
    }
    X[((size_t)r * nz + zi) * n + i] = make_double2(xr, xi);
  }
}

// The same in double-float: thread per row i, kCombineZ shifts per thread (V[k][i] read once
// for all of them), sums in double-float, FP64 only for the output.
constexpr int kCombineZ = 8;
__global__ void __launch_bounds__(128) combine_df_kernel(const float4* __restrict__ V, const float4* __restrict__ coef,
                                                         const int32_t* __restrict__ m_arr, int64_t n, int nz,
                                                         int k_cap, double2* __restrict__ X) {
  const int r = blockIdx.z;
  const int z0 = blockIdx.y * kCombineZ;
  const int m = m_arr[r];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const float4* c = coef + (size_t)r * k_cap * nz;
  const float4* Vr = V + (size_t)r * k_cap * n;
  dacc xr[kCombineZ], xi[kCombineZ];
#pragma unroll
  for (int u = 0; u < kCombineZ; ++u) xr[u] = xi[u] = {0.f, 0.f};
  if (i < n) {
    for (int k = 0; k < m; ++k) {
      const float4 v = Vr[(size_t)k * n + i];
#pragma unroll
      for (int u = 0; u < kCombineZ; ++u) {
        const float4 ck = z0 + u < nz ? __ldg(c + (size_t)k * nz + z0 + u) : make_float4(0.f, 0.f, 0.f, 0.f);
        const dfl cr = {ck.x, ck.y}, ci = {ck.z, ck.w}, nci = {-ck.z, -ck.w};
        dacc_fma(xr[u], cr, v.x, v.y);
        dacc_fma(xr[u], nci, v.z, v.w);
        dacc_fma(xi[u], cr, v.z, v.w);
        dacc_fma(xi[u], ci, v.x, v.y);
      }
    }
#pragma unroll
    for (int u = 0; u < kCombineZ; ++u)
      if (z0 + u < nz) X[((size_t)r * nz + z0 + u) * n + i] = make_double2(df_val(dacc_val(xr[u])), df_val(dacc_val(xi[u])));
  }
}

}  // namespace edgpu

extern "C" size_t edgpu_shifted_solve_workspace(int64_t n, int n_rhs, int nz, int k_cap) {
  size_t b = 0;
  b += sizeof(double2) * (size_t)n_rhs * k_cap * n + 256;       // V
  b += 2 * sizeof(double) * (size_t)n_rhs * k_cap + 512;        // alpha, beta
  b += sizeof(int32_t) * (size_t)n_rhs + sizeof(double) * n_rhs + 512;
  b += 3 * sizeof(double2) * (size_t)n_rhs * nz * k_cap + 768;  // coefficients + Thomas scratch
  return b + 1024;
}

namespace {

int shifted_solve_impl(const edgpu_csr* h, const double* Y, int n_rhs, const double* zs, int nz, int k_cap, double tol,
                       double* X, int32_t* m_out, int32_t* status_dev, void* workspace, size_t workspace_bytes,
                       cudaStream_t s, bool df) {
  using namespace edgpu;
  if (!h || !Y || !zs || !X || !m_out || !status_dev || n_rhs < 1 || nz < 1 || k_cap < 1 || h->n < 1)
    return EDGPU_ERR_ARG;
  if (nz > kSmallThreads) return EDGPU_ERR_ARG;
  if (df && (!h->val_df || h->val_c)) return EDGPU_ERR_ARG;
  if (workspace_bytes < edgpu_shifted_solve_workspace(h->n, n_rhs, nz, k_cap)) return EDGPU_ERR_WORKSPACE;
  const int64_t n = h->n;
  const size_t smem = df ? small_smem_bytes(n, 3) : 3 * sizeof(double2) * (size_t)n + 34 * sizeof(double) + 16;
  if (smem > 200 * 1024) return EDGPU_ERR_ARG;
  const size_t coef_smem = 2 * sizeof(double) * (size_t)k_cap;
  if (coef_smem > 200 * 1024) return EDGPU_ERR_ARG;
  unsigned char* ws = reinterpret_cast<unsigned char*>(workspace);
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    unsigned char* p = ws + off;
    off += (bytes + 255) & ~(size_t)255;
    return p;
  };
  void* V = carve(sizeof(double2) * (size_t)n_rhs * k_cap * n);
  double* alpha = reinterpret_cast<double*>(carve(sizeof(double) * (size_t)n_rhs * k_cap));
  double* beta = reinterpret_cast<double*>(carve(sizeof(double) * (size_t)n_rhs * k_cap));
  double* yn = reinterpret_cast<double*>(carve(sizeof(double) * (size_t)n_rhs));
  const size_t cbytes = sizeof(double2) * (size_t)n_rhs * nz * k_cap;
  void* coef = carve(cbytes);
  double2* cp = reinterpret_cast<double2*>(carve(cbytes));
  double2* xs = reinterpret_cast<double2*>(carve(cbytes));
  if (off > workspace_bytes) return EDGPU_ERR_WORKSPACE;
  const double2* Yc = reinterpret_cast<const double2*>(Y);
  const double2* zc = reinterpret_cast<const double2*>(zs);
  int per_sm = 0;
  if (df) {
    auto kern = shifted_small_df_kernel<kSmallThreads>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSmallThreads, smem);
    if (per_sm < 1) per_sm = 1;
    const int grid = std::min(grid_cap() * per_sm, n_rhs);
    kern<<<grid, kSmallThreads, smem, s>>>(n, h->row_ptr, h->col, reinterpret_cast<const float2*>(h->val_df), n_rhs,
                                           Yc, zc, nz, k_cap, (float)tol, reinterpret_cast<float4*>(V), alpha, beta,
                                           m_out, yn, status_dev);
  } else {
    auto kern = h->val_c ? shifted_small_kernel<true> : shifted_small_kernel<false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSmallThreads, smem);
    if (per_sm < 1) per_sm = 1;
    const int grid = std::min(grid_cap() * per_sm, n_rhs);
    kern<<<grid, kSmallThreads, smem, s>>>(n, h->row_ptr, h->col, h->val_c ? h->val_c : h->val_r, n_rhs, Yc, zc, nz,
                                           k_cap, tol, reinterpret_cast<double2*>(V), alpha, beta, m_out, yn,
                                           status_dev);
  }
  note_launch();
  int rc = check_launch();
  if (rc) return rc;
  const int cthreads = nz < 128 ? ((nz + 31) / 32) * 32 : 128;
  if (df) {
    cudaFuncSetAttribute(shifted_coef_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)coef_smem);
    shifted_coef_kernel<true><<<n_rhs, cthreads, coef_smem, s>>>(alpha, beta, m_out, yn, zc, nz, k_cap, nullptr,
                                                                 reinterpret_cast<float4*>(coef), cp, xs);
  } else {
    cudaFuncSetAttribute(shifted_coef_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)coef_smem);
    shifted_coef_kernel<false><<<n_rhs, cthreads, coef_smem, s>>>(alpha, beta, m_out, yn, zc, nz, k_cap,
                                                                  reinterpret_cast<double2*>(coef), nullptr, cp, xs);
  }
  note_launch();
  if (df) {
    dim3 g3((unsigned)((n + 127) / 128), (unsigned)((nz + kCombineZ - 1) / kCombineZ), (unsigned)n_rhs);
    combine_df_kernel<<<g3, 128, 0, s>>>(reinterpret_cast<const float4*>(V), reinterpret_cast<const float4*>(coef), m_out,
                                         n, nz, k_cap, reinterpret_cast<double2*>(X));
  } else {
    dim3 g3((unsigned)((n + 255) / 256 > 16 ? 16 : (n + 255) / 256), nz, n_rhs);
    combine_batched_kernel<<<g3, 256, 0, s>>>(reinterpret_cast<const double2*>(V),
                                              reinterpret_cast<const double2*>(coef), m_out, n, nz, k_cap,
                                              reinterpret_cast<double2*>(X));
  }
  note_launch();
  return check_launch();
}

}  // namespace

extern "C" int edgpu_shifted_solve(const edgpu_csr* h, const double* Y, int n_rhs, const double* zs, int nz, int k_cap,
                                   double tol, double* X, int32_t* m_out, int32_t* status_dev, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  return shifted_solve_impl(h, Y, n_rhs, zs, nz, k_cap, tol, X, m_out, status_dev, workspace, workspace_bytes,
                            (cudaStream_t)stream, false);
}

extern "C" int edgpu_shifted_solve_df(const edgpu_csr* h, const double* Y, int n_rhs, const double* zs, int nz,
                                      int k_cap, double tol, double* X, int32_t* m_out, int32_t* status_dev,
                                      void* workspace, size_t workspace_bytes, void* stream) {
  return shifted_solve_impl(h, Y, n_rhs, zs, nz, k_cap, tol, X, m_out, status_dev, workspace, workspace_bytes,
                            (cudaStream_t)stream, true);
}

// =======================================================================================
// Allocation-free batched Lanczos (edgpu_lanczos_noalloc).
//
// For callers that cannot allocate device memory themselves.  The grid-wide batched
// Lanczos needs three [n][R] vectors and per-block partial sums as scratch; here that
// scratch is this file's static device array, which every GPU that loads the library
// holds until the process exits.  Host code must not hand the array's name to a kernel
// (in host code it is only a stand-in symbol): its device address is looked up once per
// device with cudaGetSymbolAddress, with that device current, and cached.
// =======================================================================================
#include <mutex>

static __device__ __align__(256) unsigned char g_lanczos_noalloc_scratch[EDGPU_LANCZOS_NOALLOC_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kMaxDevices] = {};

int noalloc_scratch_address(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return EDGPU_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return EDGPU_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_lanczos_noalloc_scratch) != cudaSuccess || !p) return EDGPU_ERR_CUDA;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return EDGPU_OK;
}
}  // namespace

extern "C" int edgpu_lanczos_noalloc(const edgpu_csr* h, const double* v0, int R, const int32_t* k_max, int K,
                                     int precision, double* alpha, double* beta, int32_t* status_dev, void* stream) {
  if (!h || !v0 || R < 1 || K < 1 || !k_max || !alpha || !beta || !status_dev || h->n < 1) return EDGPU_ERR_ARG;
  // the same precision values as edgpu_lanczos accepts
  if (precision < 0 || precision > 3 || precision == 2) return EDGPU_ERR_ARG;
  if (precision == 3) precision = 0;  // the df64 form has no grid-wide variant
  if (precision == 0 && !h->val_c && !h->val_r) return EDGPU_ERR_ARG;
  if (precision != 0 && !h->val_cf && !h->val_rf) return EDGPU_ERR_ARG;
  if (edgpu_lanczos_workspace(h->n, R, K, precision) > (size_t)EDGPU_LANCZOS_NOALLOC_BYTES)
    return EDGPU_ERR_WORKSPACE;
  void* scratch = nullptr;
  const int rc = noalloc_scratch_address(&scratch);
  if (rc) return rc;
  unsigned char* ws = reinterpret_cast<unsigned char*>(scratch);
  const size_t bytes = (size_t)EDGPU_LANCZOS_NOALLOC_BYTES;
  cudaStream_t s = (cudaStream_t)stream;
  // Every buffer in the scratch is written before it is read (the start vectors are
  // copied in, v_{j-1} is first read after step 0 wrote it, partial sums are written by
  // the kernel that precedes their reader), so nothing has to be cleared between calls.
  if (precision == 0) return edgpu::lanczos_impl<double>(h, v0, R, k_max, K, alpha, beta, status_dev, ws, bytes, s);
  return edgpu::lanczos_impl<float>(h, v0, R, k_max, K, alpha, beta, status_dev, ws, bytes, s);
}

extern "C" size_t edgpu_lanczos_noalloc_bytes(void) { return (size_t)EDGPU_LANCZOS_NOALLOC_BYTES; }

extern "C" void edgpu_lanczos_noalloc_forget(void) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  for (int d = 0; d < kMaxDevices; ++d) g_noalloc_ptr[d] = nullptr;
}
