// Lanczos with full reorthogonalisation as one cooperative (grid-wide persistent) launch per
// chunk of steps.
//
// The grid-wide form issues seven launches per Krylov step (SpMV + alpha, alpha update, two
// Gram-Schmidt passes of dot + project, normalise); on the ground-state sectors of the
// 50-bath model (n = 1770, K <= 300) those launches, not bandwidth, set the cost.  Here one
// cooperative launch with one block per SM runs the same phases separated by grid barriers
// (cooperative_groups grid sync, ~1.2 us on GB300), keeping all 152 SMs' FP64 units on the
// Gram-Schmidt arithmetic (a single SM retires only ~4 GFMA/s in FP64).  Same recurrence:
//   w = H v_j, alpha_j = Re<v_j, w>, w -= alpha_j v_j + beta_{j-1} v_{j-1},
//   twice: h = V^H w, w -= V h;  beta_j = ||w||, v_{j+1} = w / beta_j.
// Scalars are summed from per-block partials in one fixed order by every block, so all
// blocks hold identical values and take identical branches around the grid barriers.
#include <cooperative_groups.h>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace edgpu {

constexpr int kCoopThreads = 256;
constexpr int kCoopMaxBlocks = 1024;
constexpr int64_t kCoopMaxN = 65536;

size_t reorth_coop_scratch_bytes() { return 2 * sizeof(double) * kCoopMaxBlocks; }

// Deterministic block reduction; the result is valid in thread 0 only.
__device__ __forceinline__ double coop_block_sum0(double v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
  return t;
}

// Sum of p[0..cnt) in one fixed order (lane-strided, then an xor tree), returned to every
// thread of the block; identical bits in every block.
__device__ __forceinline__ double coop_fixed_sum(const double* p, int cnt, double* bcast) {
  if (threadIdx.x < 32) {
    double s = 0.0;
    for (int q = threadIdx.x; q < cnt; q += 32) s += p[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) *bcast = s;
  }
  __syncthreads();
  const double s = *bcast;
  __syncthreads();
  return s;
}

template <bool VALC>
__global__ void __launch_bounds__(kCoopThreads)
    lanczos_reorth_coop_kernel(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                               const double* __restrict__ vals, const double2* __restrict__ v0, int j0, int j1,
                               int K_cap, double2* V, double2* w, double* alpha, double* beta, int32_t* status,
                               double* pa, double* pn, double2* hc) {
  cg::grid_group grid = cg::this_grid();
  const int B = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31;
  const int64_t gtid = (int64_t)b * blockDim.x + tid, gthreads = (int64_t)B * blockDim.x;
  __shared__ double red[33];
  __shared__ double bc;
  __shared__ double2 part[8][32];

  if (j0 == 0)
    for (int64_t i = gtid; i < n; i += gthreads) V[i] = v0[i];
  double bprev = (j0 > 0) ? beta[j0 - 1] : 0.0;
  grid.sync();

  for (int j = j0; j < j1; ++j) {
    const double2* vj = V + (int64_t)j * n;
    const double2* vjm1 = j > 0 ? V + (int64_t)(j - 1) * n : nullptr;
    // w = H v_j: 8 lanes per row (every 8th entry each), fixed xor tree; alpha partials
    double ap = 0.0;
    const int sub = (int)(gtid & 7);
    for (int64_t rb = 0; rb < n; rb += gthreads >> 3) {
      const int64_t i = rb + (gtid >> 3);
      double yr = 0.0, yi = 0.0;
      if (i < n) {
        const int64_t e1 = rp[i + 1];
        for (int64_t e = rp[i] + sub; e < e1; e += 8) {
          const double2 x = vj[col[e]];
          if (VALC) {
            const double hr = vals[2 * e], hm = vals[2 * e + 1];
            yr += hr * x.x - hm * x.y;
            yi += hr * x.y + hm * x.x;
          } else {
            const double hr = vals[e];
            yr += hr * x.x;
            yi += hr * x.y;
          }
        }
      }
#pragma unroll
      for (int o = 4; o > 0; o >>= 1) {
        yr += __shfl_xor_sync(0xffffffffu, yr, o);
        yi += __shfl_xor_sync(0xffffffffu, yi, o);
      }
      if (sub == 0 && i < n) {
        const double2 v = vj[i];
        ap += v.x * yr + v.y * yi;
        w[i] = make_double2(yr, yi);
      }
    }
    ap = coop_block_sum0(ap, red);
    if (tid == 0) pa[b] = ap;
    grid.sync();
    const double a = coop_fixed_sum(pa, B, &bc);
    for (int64_t i = gtid; i < n; i += gthreads) {
      double2 y = w[i];
      const double2 c = vj[i];
      y.x -= a * c.x;
      y.y -= a * c.y;
      if (j > 0) {
        const double2 p = vjm1[i];
        y.x -= bprev * p.x;
        y.y -= bprev * p.y;
      }
      w[i] = y;
    }
    if (b == 0 && tid == 0) alpha[j] = a;
    if (j + 1 >= K_cap) break;
    grid.sync();
    // two passes of classical Gram-Schmidt against V[0..j]
    const int m = j + 1;
    double nrm = 0.0;
    for (int pass = 0; pass < 2; ++pass) {
      // h_k = <v_k, w>: one block per k over all rows
      for (int k = b; k < m; k += B) {
        const double2* vk = V + (int64_t)k * n;
        double hr = 0.0, hm = 0.0, gr = 0.0, gm = 0.0;
        int64_t i = tid;
        for (; i + kCoopThreads < n; i += 2 * kCoopThreads) {
          const double2 v1 = vk[i], x1 = w[i], v2 = vk[i + kCoopThreads], x2 = w[i + kCoopThreads];
          hr += v1.x * x1.x + v1.y * x1.y;
          hm += v1.x * x1.y - v1.y * x1.x;
          gr += v2.x * x2.x + v2.y * x2.y;
          gm += v2.x * x2.y - v2.y * x2.x;
        }
        for (; i < n; i += kCoopThreads) {
          const double2 v1 = vk[i], x1 = w[i];
          hr += v1.x * x1.x + v1.y * x1.y;
          hm += v1.x * x1.y - v1.y * x1.x;
        }
        const double sr = coop_block_sum0(hr + gr, red);
        const double si = coop_block_sum0(hm + gm, red);
        if (tid == 0) hc[k] = make_double2(sr, si);
      }
      grid.sync();
      // w -= V h on tiles of 32 rows x 8 k-classes
      const int ri = tid & 31, kc = tid >> 5;
      for (int64_t t0 = (int64_t)b * 32; t0 < n; t0 += (int64_t)B * 32) {
        const int64_t i = t0 + ri;
        double2 acc = make_double2(0.0, 0.0);
        if (i < n) {
#pragma unroll 4
          for (int k = kc; k < m; k += 8) {
            const double2 c = hc[k];
            const double2 v = V[(int64_t)k * n + i];
            acc.x += c.x * v.x - c.y * v.y;
            acc.y += c.x * v.y + c.y * v.x;
          }
        }
        part[kc][ri] = acc;
        __syncthreads();
        if (kc == 0 && i < n) {
          double2 x = w[i];
          for (int q = 0; q < 8; ++q) {
            x.x -= part[q][ri].x;
            x.y -= part[q][ri].y;
          }
          w[i] = x;
          if (pass == 1) nrm += x.x * x.x + x.y * x.y;
        }
        __syncthreads();
      }
      if (pass == 1) {
        nrm = coop_block_sum0(nrm, red);
        if (tid == 0) pn[b] = nrm;
      }
      grid.sync();
    }
    const double bt = sqrt(coop_fixed_sum(pn, B, &bc));
    if (b == 0 && tid == 0) {
      beta[j] = bt;
      if (!(bt > 0.0)) atomicExch(status, (int32_t)(bt == 0.0 ? EDGPU_ERR_BREAKDOWN : EDGPU_ERR_NAN));
    }
    if (!(bt > 0.0)) break;  // identical in every block
    double2* vn = V + (int64_t)(j + 1) * n;
    for (int64_t i = gtid; i < n; i += gthreads) {
      const double2 y = w[i];
      vn[i] = make_double2(y.x / bt, y.y / bt);
    }
    bprev = bt;
    grid.sync();  // v_{j+1} complete before the next SpMV gathers it
  }
  (void)lane;
}

// Returns -1 when the sector is outside the cooperative kernel's range or the device cannot
// co-schedule the grid (caller uses the per-step kernels), else a status.
int lanczos_reorth_coop(const edgpu_csr* h, const double* v0, int j0, int j1, int K_cap, double* Vd, double* wd,
                        double* alpha, double* beta, int32_t* status_dev, double* scratch, double2* hc,
                        cudaStream_t s) {
  if (h->n > kCoopMaxN || (!h->val_c && !h->val_r)) return -1;
  int dev = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) {
    cudaGetLastError();
    return -1;
  }
  void (*kern)(int64_t, const int64_t*, const int32_t*, const double*, const double2*, int, int, int, double2*,
               double2*, double*, double*, int32_t*, double*, double*, double2*) =
      h->val_c ? lanczos_reorth_coop_kernel<true> : lanczos_reorth_coop_kernel<false>;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCoopThreads, 0) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    return -1;
  }
  int blocks = grid_cap();  // one block per SM: enough threads for these sectors, cheapest barrier
  if (blocks > kCoopMaxBlocks) blocks = kCoopMaxBlocks;
  int64_t n = h->n;
  const int64_t* rp = h->row_ptr;
  const int32_t* col = h->col;
  const double* vals = h->val_c ? h->val_c : h->val_r;
  const double2* v0c = reinterpret_cast<const double2*>(v0);
  double2* V = reinterpret_cast<double2*>(Vd);
  double2* w = reinterpret_cast<double2*>(wd);
  double* pa = scratch;
  double* pn = scratch + kCoopMaxBlocks;
  void* args[] = {&n, &rp, &col, &vals, &v0c, &j0, &j1, &K_cap, &V, &w, &alpha, &beta, &status_dev, &pa, &pn, &hc};
  const cudaError_t e = cudaLaunchCooperativeKernel((const void*)kern, blocks, kCoopThreads, args, 0, s);
  note_launch();
  if (e != cudaSuccess) {
    cudaGetLastError();
    return EDGPU_ERR_CUDA;
  }
  return check_launch();
}

}  // namespace edgpu
