// Ragged batches: sectors of different sizes (an ensemble of models, each with its own
// Hamiltonian) concatenated into one CSR and solved in one launch with one CTA per run.
//
// Layout: rows of sector s are [sec_row0[s], sec_row0[s+1]) of the concatenated row_ptr;
// column indices are local to the sector (0 .. n_s - 1).  Run r works on sector run_sec[r];
// its vectors live at offset run_vec0[r] of packed [sum over runs of n] arrays.
//
// Upstream counterparts: get_tridiagonal_krylov_vectors (impurityModel/ed/finite.py:1897-1995)
// per run for the spectra, and the eigsh call of eigensystem (finite.py:105) per model for the
// ground states (Lanczos with full reorthogonalisation here, as in edgpu_lanczos_reorth).
#include "common.cuh"

namespace edgpu {

constexpr int kRaggedThreads = 512;

// Deterministic block sum, broadcast to every thread.
__device__ __forceinline__ double rg_block_sum(double v, double* red) {
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
  const double s = red[32];
  __syncthreads();
  return s;
}

// y = H x on a sector's rows (thread-strided), x and y in shared memory.
template <bool VALC>
__device__ __forceinline__ double rg_spmv_alpha(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                                const double* __restrict__ vals, int64_t n, const double2* x,
                                                double2* y) {
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    double yr = 0.0, yi = 0.0;
    const int64_t e1 = rp[i + 1];
    for (int64_t e = rp[i]; e < e1; ++e) {
      const double2 xv = x[col[e]];
      if (VALC) {
        const double hr = vals[2 * e], hm = vals[2 * e + 1];
        yr += hr * xv.x - hm * xv.y;
        yi += hr * xv.y + hm * xv.x;
      } else {
        const double h = vals[e];
        yr += h * xv.x;
        yi += h * xv.y;
      }
    }
    y[i] = make_double2(yr, yi);
    const double2 xi = x[i];
    acc += yr * xi.x + yi * xi.y;
  }
  return acc;
}

// Upstream's recurrence (no reorthogonalisation), one CTA per run, three vectors in shared
// memory; same arithmetic order as lanczos_small_kernel<double>.
template <bool VALC>
__global__ void __launch_bounds__(kRaggedThreads)
    lanczos_ragged_kernel(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                          const double* __restrict__ vals, const int64_t* __restrict__ sec_row0,
                          const int32_t* __restrict__ run_sec, const int64_t* __restrict__ run_vec0, int R,
                          const double2* __restrict__ v0, const int32_t* __restrict__ k_max, int K,
                          int64_t max_rows, double* __restrict__ alpha, double* __restrict__ beta, int32_t* status) {
  extern __shared__ __align__(16) unsigned char sm[];
  double2* A = reinterpret_cast<double2*>(sm);
  double2* B = A + max_rows;
  double2* Cv = B + max_rows;
  double* red = reinterpret_cast<double*>(Cv + max_rows);
  const int tid = threadIdx.x, bs = blockDim.x;
  for (int r = blockIdx.x; r < R; r += gridDim.x) {
    const int km = k_max[r];
    const int s = run_sec[r];
    const int64_t row0 = sec_row0[s];
    const int64_t n = sec_row0[s + 1] - row0;
    if (n > max_rows) {
      if (tid == 0) atomicExch(status, (int32_t)EDGPU_ERR_WORKSPACE);
      continue;
    }
    if (km <= 0 || n <= 0) continue;
    const int64_t* rps = rp + row0;
    const double2* vr = v0 + run_vec0[r];
    for (int64_t i = tid; i < n; i += bs) {
      A[i] = vr[i];
      B[i] = make_double2(0.0, 0.0);
    }
    __syncthreads();
    double2* x = A;
    double2* p = B;
    double2* y = Cv;
    double bprev = 0.0;
    for (int j = 0; j < km; ++j) {
      const double a = rg_block_sum(rg_spmv_alpha<VALC>(rps, col, vals, n, x, y), red);
      if (tid == 0) alpha[(int64_t)r * K + j] = a;
      if (j + 1 == km) break;
      double acc = 0.0;
      for (int64_t i = tid; i < n; i += bs) {
        double2 w = y[i];
        const double2 xi = x[i], pi = p[i];
        w.x = (w.x - a * xi.x) - bprev * pi.x;
        w.y = (w.y - a * xi.y) - bprev * pi.y;
        y[i] = w;
        acc += w.x * w.x + w.y * w.y;
      }
      const double b = sqrt(rg_block_sum(acc, red));
      if (tid == 0) {
        beta[(int64_t)r * K + j] = b;
        if (!(b > 0.0)) atomicExch(status, (int32_t)(b == 0.0 ? EDGPU_ERR_BREAKDOWN : EDGPU_ERR_NAN));
      }
      const double inv = b > 0.0 ? 1.0 / b : 0.0;
      for (int64_t i = tid; i < n; i += bs) {
        const double2 w = y[i];
        p[i] = make_double2(w.x * inv, w.y * inv);  // v_{j-1}'s buffer becomes v_{j+1}
      }
      __syncthreads();
      double2* t = p;
      p = x;
      x = t;
      bprev = b;
    }
    __syncthreads();
  }
}

// Lanczos with full reorthogonalisation (classical Gram-Schmidt, a second pass where the DGKS
// test asks), one CTA per run;
// the Krylov basis of run r at V + run_V0[r] ([k_max[r]][n] complex128), the work vector and
// projections in shared memory.  beta[r][k_max-1] is the residual coupling of the last step
// (for Ritz residual estimates); no vector is formed from it.
template <bool VALC>
__global__ void __launch_bounds__(kRaggedThreads)
    lanczos_reorth_ragged_kernel(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                 const double* __restrict__ vals, const int64_t* __restrict__ sec_row0,
                                 const int32_t* __restrict__ run_sec, const int64_t* __restrict__ run_vec0, int R,
                                 const double2* __restrict__ v0, const int32_t* __restrict__ k_max, int K,
                                 int64_t max_rows, const int64_t* __restrict__ run_V0, double2* V,
                                 double* __restrict__ alpha, double* __restrict__ beta, int32_t* status) {
  extern __shared__ __align__(16) unsigned char sm[];
  double2* w = reinterpret_cast<double2*>(sm);  // [max_rows]
  double2* h = w + max_rows;                    // [K]
  double* red = reinterpret_cast<double*>(h + K);
  const int tid = threadIdx.x, bs = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = bs >> 5;
  for (int r = blockIdx.x; r < R; r += gridDim.x) {
    const int km = k_max[r];
    const int s = run_sec[r];
    const int64_t row0 = sec_row0[s];
    const int64_t n = sec_row0[s + 1] - row0;
    if (n > max_rows || km > K) {
      if (tid == 0) atomicExch(status, (int32_t)EDGPU_ERR_WORKSPACE);
      continue;
    }
    if (km <= 0 || n <= 0) continue;
    const int64_t* rps = rp + row0;
    double2* Vr = V + run_V0[r];
    const double2* vr = v0 + run_vec0[r];
    for (int64_t i = tid; i < n; i += bs) Vr[i] = vr[i];
    __syncthreads();
    double bprev = 0.0;
    for (int j = 0; j < km; ++j) {
      const double2* vj = Vr + (int64_t)j * n;
      const double a = rg_block_sum(rg_spmv_alpha<VALC>(rps, col, vals, n, vj, w), red);
      for (int64_t i = tid; i < n; i += bs) {
        double2 y = w[i];
        const double2 c = vj[i];
        y.x -= a * c.x;
        y.y -= a * c.y;
        if (j > 0) {
          const double2 p = vj[i - n];
          y.x -= bprev * p.x;
          y.y -= bprev * p.y;
        }
        w[i] = y;
      }
      if (tid == 0) alpha[(int64_t)r * K + j] = a;
      const int m = j + 1;
      // classical Gram-Schmidt against the whole basis, a second pass only when the first
      // removed more than half of |w|^2 (the test of Daniel, Gragg, Kaufman and Stewart with
      // eta = 1/sqrt(2): |w_before|^2 = |w_after|^2 + |h|^2, so the test is |h|^2 > |w_after|^2)
      double wn = 0.0;  // |w|^2 after the last pass (block sum)
      for (int pass = 0; pass < 2; ++pass) {
        double nrm = 0.0;
        __syncthreads();
        for (int k = warp; k < m; k += nwarps) {
          const double2* vk = Vr + (int64_t)k * n;
          double hr = 0.0, hm = 0.0;
          for (int64_t i = lane; i < n; i += 32) {
            const double2 v = vk[i], x = w[i];
            hr += v.x * x.x + v.y * x.y;
            hm += v.x * x.y - v.y * x.x;
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            hr += __shfl_down_sync(0xffffffffu, hr, o);
            hm += __shfl_down_sync(0xffffffffu, hm, o);
          }
          if (lane == 0) h[k] = make_double2(hr, hm);
        }
        __syncthreads();
        for (int64_t i = tid; i < n; i += bs) {
          double2 acc = make_double2(0.0, 0.0);
#pragma unroll 4
          for (int k = 0; k < m; ++k) {
            const double2 c = h[k];
            const double2 v = Vr[(int64_t)k * n + i];
            acc.x += c.x * v.x - c.y * v.y;
            acc.y += c.x * v.y + c.y * v.x;
          }
          double2 x = w[i];
          x.x -= acc.x;
          x.y -= acc.y;
          w[i] = x;
          nrm += x.x * x.x + x.y * x.y;
        }
        wn = rg_block_sum(nrm, red);
        if (pass == 0) {
          double hh = 0.0;
          for (int k = tid; k < m; k += bs) hh += h[k].x * h[k].x + h[k].y * h[k].y;
          if (!(rg_block_sum(hh, red) > wn)) break;  // the same decision in every thread
        }
      }
      const double b = sqrt(wn);
      if (tid == 0) beta[(int64_t)r * K + j] = b;
      if (j + 1 == km) break;
      if (!(b > 0.0)) {
        if (tid == 0) atomicExch(status, (int32_t)(b == 0.0 ? EDGPU_ERR_BREAKDOWN : EDGPU_ERR_NAN));
        break;
      }
      double2* vn = Vr + (int64_t)(j + 1) * n;
      for (int64_t i = tid; i < n; i += bs) {
        const double2 y = w[i];
        vn[i] = make_double2(y.x / b, y.y / b);
      }
      bprev = b;
      __syncthreads();
    }
    __syncthreads();
  }
}

// X[r][q] = sum_k S[r][k][q] V_r[k] for q < Q (Ritz vectors), packed at Q * run_vec0[r].
__global__ void combine_ragged_kernel(const double2* __restrict__ V, const int64_t* __restrict__ sec_row0,
                                      const int32_t* __restrict__ run_sec, const int64_t* __restrict__ run_vec0,
                                      const int64_t* __restrict__ run_V0, const int32_t* __restrict__ k_len,
                                      const double* __restrict__ S, int K, int Q, double2* __restrict__ X) {
  const int r = blockIdx.x, q = blockIdx.y;
  const int s = run_sec[r];
  const int64_t n = sec_row0[s + 1] - sec_row0[s];
  const int kl = k_len[r];
  const double2* Vr = V + run_V0[r];
  const double* Sr = S + (int64_t)r * K * Q;
  double2* Xr = X + (int64_t)Q * run_vec0[r] + (int64_t)q * n;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    double xr = 0.0, xi = 0.0;
    for (int k = 0; k < kl; ++k) {
      const double c = Sr[(int64_t)k * Q + q];
      const double2 v = Vr[(int64_t)k * n + i];
      xr += c * v.x;
      xi += c * v.y;
    }
    Xr[i] = make_double2(xr, xi);
  }
}

namespace {
bool ragged_ok(const edgpu_csr* h, const edgpu_ragged* rg) {
  return h && rg && rg->n_runs >= 0 && rg->n_sectors >= 1 && rg->sec_row0 && rg->run_sec && rg->run_vec0 &&
         rg->max_rows >= 1 && (h->val_c || h->val_r);
}
}  // namespace

}  // namespace edgpu

using namespace edgpu;

extern "C" size_t edgpu_lanczos_ragged_smem(int64_t max_rows) {
  return 3 * sizeof(double2) * (size_t)max_rows + 34 * sizeof(double) + 16;
}

extern "C" size_t edgpu_lanczos_reorth_ragged_smem(int64_t max_rows, int K) {
  return sizeof(double2) * ((size_t)max_rows + (size_t)K) + 34 * sizeof(double) + 16;
}

extern "C" int edgpu_lanczos_ragged(const edgpu_csr* h, const edgpu_ragged* rg, const double* v0,
                                    const int32_t* k_max, int K, double* alpha, double* beta, int32_t* status_dev,
                                    void* stream) {
  if (!ragged_ok(h, rg) || !v0 || !k_max || K < 1 || !alpha || !beta || !status_dev) return EDGPU_ERR_ARG;
  if (rg->n_runs == 0) return EDGPU_OK;
  const size_t smem = edgpu_lanczos_ragged_smem(rg->max_rows);
  if (smem > 200 * 1024) return EDGPU_ERR_ARG;
  auto* kern = h->val_c ? lanczos_ragged_kernel<true> : lanczos_ragged_kernel<false>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kRaggedThreads, smem);
  if (per_sm < 1) per_sm = 1;
  int grid = grid_cap() * per_sm;
  if (grid > rg->n_runs) grid = rg->n_runs;
  kern<<<grid, kRaggedThreads, smem, (cudaStream_t)stream>>>(
      h->row_ptr, h->col, h->val_c ? h->val_c : h->val_r, rg->sec_row0, rg->run_sec, rg->run_vec0, rg->n_runs,
      reinterpret_cast<const double2*>(v0), k_max, K, rg->max_rows, alpha, beta, status_dev);
  note_launch();
  return check_launch();
}

extern "C" int edgpu_lanczos_reorth_ragged(const edgpu_csr* h, const edgpu_ragged* rg, const double* v0,
                                           const int32_t* k_max, int K, const int64_t* run_V0, double* V,
                                           double* alpha, double* beta, int32_t* status_dev, void* stream) {
  if (!ragged_ok(h, rg) || !v0 || !k_max || K < 1 || !run_V0 || !V || !alpha || !beta || !status_dev)
    return EDGPU_ERR_ARG;
  if (rg->n_runs == 0) return EDGPU_OK;
  const size_t smem = edgpu_lanczos_reorth_ragged_smem(rg->max_rows, K);
  if (smem > 200 * 1024) return EDGPU_ERR_ARG;
  auto* kern = h->val_c ? lanczos_reorth_ragged_kernel<true> : lanczos_reorth_ragged_kernel<false>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kRaggedThreads, smem);
  if (per_sm < 1) per_sm = 1;
  int grid = grid_cap() * per_sm;
  if (grid > rg->n_runs) grid = rg->n_runs;
  kern<<<grid, kRaggedThreads, smem, (cudaStream_t)stream>>>(
      h->row_ptr, h->col, h->val_c ? h->val_c : h->val_r, rg->sec_row0, rg->run_sec, rg->run_vec0, rg->n_runs,
      reinterpret_cast<const double2*>(v0), k_max, K, rg->max_rows, run_V0, reinterpret_cast<double2*>(V), alpha,
      beta, status_dev);
  note_launch();
  return check_launch();
}

extern "C" int edgpu_combine_ragged(const double* V, const edgpu_ragged* rg, const int64_t* run_V0,
                                    const int32_t* k_len, const double* S, int K, int Q, double* X, void* stream) {
  if (!rg || !rg->sec_row0 || !rg->run_sec || !rg->run_vec0 || !V || !run_V0 || !k_len || !S || K < 1 || Q < 1 ||
      !X)
    return EDGPU_ERR_ARG;
  if (rg->n_runs == 0) return EDGPU_OK;
  dim3 grid(rg->n_runs, Q);
  combine_ragged_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const double2*>(V), rg->sec_row0, rg->run_sec, rg->run_vec0, run_V0, k_len, S, K, Q,
      reinterpret_cast<double2*>(X));
  note_launch();
  return check_launch();
}
