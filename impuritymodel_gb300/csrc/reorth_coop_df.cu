// Lanczos with full reorthogonalisation in double-float arithmetic, one cooperative launch
// per chunk of steps, for a real H with its hi/lo float copy (val_df).
//
// The recurrence of lanczos_reorth_coop_kernel (upstream's eigensystem replaced by Ritz pairs
// of the reorthogonalised Krylov space):
//   w = H v_j, alpha_j = Re<v_j, w>, w -= alpha_j v_j + beta_{j-1} v_{j-1},
//   twice: h = V^H w, w -= V h;  beta_j = ||w||, v_{j+1} = w / beta_j,
// with vectors stored as float4 (re.hi, re.lo, im.hi, im.lo) and every multiply-add on the
// FP32 pipe (GB300 retires FP64 at 1/64 of the FP32 rate; in FP64 the Gram-Schmidt dots and
// projections, not the barriers, set the cost of a step).  Five grid barriers per step:
//   A   y = H v_j (8 lanes per row), where v_j = w / beta_{j-1} is formed on the fly and
//       written to V[j] by the row's first lane; partials of alpha_j.
//   C1  alpha_j from the partials; w' = y - alpha_j v_j - beta_{j-1} v_{j-1} stored into w
//       (grid stride) and recomputed on the fly for the dots h_k = <v_k, w'> (block per k).
//   D1  w -= V h on tiles of 16 rows x 64 k-classes (a warp: 16 rows x 2 k-classes).
//   C2  h_k = <v_k, w>.
//   D2  w -= V h, partials of |w|^2.
// C1 and D1 also sum |w'|^2 and |w|^2; the second pass (C2, D2) runs only when the first one
// removed more than half of |w'|^2 (Kahan's "twice is enough" test: after a pass that keeps
// |w| >= |w'| / sqrt(2), w is orthogonal to V to working precision).  In a Lanczos step w'
// is already orthogonal to V up to rounding, so the second pass is normally skipped and a
// step takes three grid barriers.
// Every block sums the per-block partials in one fixed order, so all blocks hold identical
// alpha, beta and take identical branches; beta_j is formed after D2's barrier and v_{j+1} is
// materialised by the next step's gather (also across chunk launches: w and beta persist).
#include <cooperative_groups.h>

#include "common.cuh"
#include "df64.cuh"

namespace cg = cooperative_groups;

namespace edgpu {

// One 1024-thread block per SM: each phase is a few dependent L2 round trips per thread, so
// the 32 warps are what hides their latency.
constexpr int kCoopDfThreads = 1024;
constexpr int kCoopDfWarps = kCoopDfThreads / 32;
constexpr int kCoopDfMaxBlocks = 1024;
constexpr int64_t kCoopDfMaxN = 65536;
// A block's gather rows (blockDim / 8 of them) and their CSR entries are cached in shared
// memory when the sector is gathered in one pass and the block's rows hold at most this
// many entries: each step then needs one L2 round trip (the x gather) instead of three.
constexpr int kCacheRows = kCoopDfThreads / 8;
constexpr int kCacheNnz = 4096;
constexpr size_t kCacheBytes = sizeof(int32_t) * (kCacheRows + 1) + (sizeof(int32_t) + sizeof(float2)) * kCacheNnz;

// Sum of the per-block partials p[0..cnt) (cnt <= blockDim.x), one per thread so that a
// single L2 round trip fetches them all, then the fixed block tree: identical bits in every
// block.  Uses the partial buffer buf like df_block_sum2.
__device__ __forceinline__ dfl coop_fixed_sum_df(const dfl* p, int cnt, dfl* buf) {
  const dfl v = (int)threadIdx.x < cnt ? p[threadIdx.x] : dfl{0.f, 0.f};
  return df_block_sum2<kCoopDfWarps>(v, buf);
}

__device__ __forceinline__ float4 df4(dfl re, dfl im) { return make_float4(re.hi, re.lo, im.hi, im.lo); }

// y - alpha v - beta p for one complex element (p absent at j = 0)
__device__ __forceinline__ float4 three_term(float4 y, float4 v, const float4* p, dfl na, dfl nb) {
  dfl r = df_fma({y.x, y.y}, na, {v.x, v.y});
  dfl m = df_fma({y.z, y.w}, na, {v.z, v.w});
  if (p) {
    const float4 q = *p;
    r = df_fma(r, nb, {q.x, q.y});
    m = df_fma(m, nb, {q.z, q.w});
  }
  return df4(r, m);
}

// acc += conj(v) * x
__device__ __forceinline__ void dot_acc(dacc& hr, dacc& hm, float4 v, float4 x) {
  dacc_fma(hr, {v.x, v.y}, x.x, x.y);
  dacc_fma(hr, {v.z, v.w}, x.z, x.w);
  dacc_fma(hm, {v.x, v.y}, x.z, x.w);
  dacc_fma(hm, {-v.z, -v.w}, x.x, x.y);
}

__global__ void __launch_bounds__(kCoopDfThreads)
    lanczos_reorth_coop_df_kernel(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                  const float2* __restrict__ hv, const double2* __restrict__ v0, int j0, int j1,
                                  int K_cap, float4* V, float4* w, float4* y, double* alpha, double* beta,
                                  int32_t* status, dfl* pa, dfl* pn, dfl* pw, float4* hc) {
  cg::grid_group grid = cg::this_grid();
  const int B = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int64_t gtid = (int64_t)b * kCoopDfThreads + tid, gthreads = (int64_t)B * kCoopDfThreads;
  __shared__ dfl red[kDfRed];
  extern __shared__ __align__(16) unsigned char dsm[];
  float2* shv = reinterpret_cast<float2*>(dsm);
  int32_t* scol = reinterpret_cast<int32_t*>(shv + kCacheNnz);
  int32_t* srp = scol + kCacheNnz;
  __shared__ float4 part[kCoopDfWarps][17];

  if (j0 == 0)
    for (int64_t i = gtid; i < n; i += gthreads) {
      const double2 v = v0[i];
      V[i] = df4(df_split(v.x), df_split(v.y));
    }
  dfl bprev = j0 > 0 ? df_split(beta[j0 - 1]) : dfl{0.f, 0.f};
  // this block's gather rows [r0, r1) when every row is gathered in the first pass
  const int64_t r0 = (int64_t)b * kCacheRows, r1 = r0 + kCacheRows < n ? r0 + kCacheRows : n;
  bool cached = false;
  if (n <= (gthreads >> 3) && r0 < n) {
    const int64_t e0 = rp[r0], ne = rp[r1] - e0;
    if (ne <= kCacheNnz) {
      cached = true;
      for (int64_t r = tid; r <= r1 - r0; r += kCoopDfThreads) srp[r] = (int32_t)(rp[r0 + r] - e0);
      for (int64_t e = tid; e < ne; e += kCoopDfThreads) {
        scol[e] = col[e0 + e];
        shv[e] = hv[e0 + e];
      }
    }
  }
  grid.sync();

  // w -= sum_k hc[k] v_k over k < m on tiles of 16 rows x 64 k-classes: lane & 15 picks the
  // row, 2 warp + (lane >> 4) the k-class; the two classes of a warp are added with one xor
  // step, then warp q < 16 sums row q over the 32 warps' partials with an xor tree.
  // Optional partial of |w|^2 (valid in thread 0).
  auto project = [&](int m, bool norm) -> dfl {
    constexpr int kRows = 16, kClasses = 2 * kCoopDfWarps;
    const int ri = lane & 15, kc = 2 * warp + (lane >> 4);
    dacc nrm = {0.f, 0.f};
    for (int64_t t0 = (int64_t)b * kRows; t0 < n; t0 += (int64_t)B * kRows) {
      const int64_t i = t0 + ri;
      dacc ar = {0.f, 0.f}, am = {0.f, 0.f};
      const int64_t iq = t0 + warp;
      float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
      if (warp < kRows && lane == 0 && iq < n) x = w[iq];  // in flight during the k loop
      if (i < n) {
        int k = kc;
        for (; k + kClasses < m; k += 2 * kClasses) {
          const float4 c1 = hc[k], c2 = hc[k + kClasses];
          const float4 v1 = V[(int64_t)k * n + i], v2 = V[(int64_t)(k + kClasses) * n + i];
          dacc_fma(ar, {c1.x, c1.y}, v1.x, v1.y);
          dacc_fma(ar, {-c1.z, -c1.w}, v1.z, v1.w);
          dacc_fma(am, {c1.x, c1.y}, v1.z, v1.w);
          dacc_fma(am, {c1.z, c1.w}, v1.x, v1.y);
          dacc_fma(ar, {c2.x, c2.y}, v2.x, v2.y);
          dacc_fma(ar, {-c2.z, -c2.w}, v2.z, v2.w);
          dacc_fma(am, {c2.x, c2.y}, v2.z, v2.w);
          dacc_fma(am, {c2.z, c2.w}, v2.x, v2.y);
        }
        if (k < m) {
          const float4 c = hc[k];
          const float4 v = V[(int64_t)k * n + i];
          dacc_fma(ar, {c.x, c.y}, v.x, v.y);
          dacc_fma(ar, {-c.z, -c.w}, v.z, v.w);
          dacc_fma(am, {c.x, c.y}, v.z, v.w);
          dacc_fma(am, {c.z, c.w}, v.x, v.y);
        }
      }
      dfl sr = dacc_val(ar), sm = dacc_val(am);
      sr = df_add(sr, {__shfl_xor_sync(0xffffffffu, sr.hi, 16), __shfl_xor_sync(0xffffffffu, sr.lo, 16)});
      sm = df_add(sm, {__shfl_xor_sync(0xffffffffu, sm.hi, 16), __shfl_xor_sync(0xffffffffu, sm.lo, 16)});
      if (lane < kRows) part[warp][lane] = df4(sr, sm);
      __syncthreads();
      if (warp < kRows) {
        const float4 s = part[lane][warp];
        dfl pr = {s.x, s.y}, pm = {s.z, s.w};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          pr = df_add(pr, {__shfl_xor_sync(0xffffffffu, pr.hi, o), __shfl_xor_sync(0xffffffffu, pr.lo, o)});
          pm = df_add(pm, {__shfl_xor_sync(0xffffffffu, pm.hi, o), __shfl_xor_sync(0xffffffffu, pm.lo, o)});
        }
        if (lane == 0 && iq < n) {
          const dfl xr = df_add({x.x, x.y}, {-pr.hi, -pr.lo});
          const dfl xm = df_add({x.z, x.w}, {-pm.hi, -pm.lo});
          w[iq] = df4(xr, xm);
          if (norm) {
            dacc_fma(nrm, xr, xr.hi, xr.lo);
            dacc_fma(nrm, xm, xm.hi, xm.lo);
          }
        }
      }
      __syncthreads();
    }
    return norm ? df_block_sum2<kCoopDfWarps>(dacc_val(nrm), red) : dfl{0.f, 0.f};
  };

  for (int j = j0; j < j1; ++j) {
    float4* vj = V + (int64_t)j * n;
    const float4* vjm1 = j > 0 ? V + (int64_t)(j - 1) * n : nullptr;
    // ---- A: y = H v_j, V[j], alpha partials
    const dfl ib = j > 0 ? df_rcp(bprev) : dfl{1.f, 0.f};
    const float4* xs = j > 0 ? w : V;
    dacc ap = {0.f, 0.f};
    const int sub = (int)(gtid & 7);
    for (int64_t rb = 0; rb < n; rb += gthreads >> 3) {
      const int64_t i = rb + (gtid >> 3);
      if (rb + ((gtid - lane) >> 3) >= n) break;  // no row for the whole warp (warp-uniform)
      dacc yr = {0.f, 0.f}, yi = {0.f, 0.f};
      float4 xi = make_float4(0.f, 0.f, 0.f, 0.f);
      if (i < n) {
        if (sub == 0) xi = xs[i];  // in flight during the gather
        if (cached) {
          const int e1 = srp[i - r0 + 1];
          for (int e = srp[i - r0] + sub; e < e1; e += 8) {
            const float2 h = shv[e];
            const float4 x = xs[scol[e]];
            dacc_fma(yr, {h.x, h.y}, x.x, x.y);
            dacc_fma(yi, {h.x, h.y}, x.z, x.w);
          }
        } else {
          const int64_t e1 = rp[i + 1];
          for (int64_t e = rp[i] + sub; e < e1; e += 8) {
            const float2 h = hv[e];
            const float4 x = xs[col[e]];
            dacc_fma(yr, {h.x, h.y}, x.x, x.y);
            dacc_fma(yi, {h.x, h.y}, x.z, x.w);
          }
        }
      }
      dfl r = dacc_val(yr), m = dacc_val(yi);
#pragma unroll
      for (int o = 4; o > 0; o >>= 1) {
        r = df_add(r, {__shfl_xor_sync(0xffffffffu, r.hi, o), __shfl_xor_sync(0xffffffffu, r.lo, o)});
        m = df_add(m, {__shfl_xor_sync(0xffffffffu, m.hi, o), __shfl_xor_sync(0xffffffffu, m.lo, o)});
      }
      if (sub == 0 && i < n) {
        float4 v = xi;
        if (j > 0) {
          r = df_mul(r, ib);
          m = df_mul(m, ib);
          v = df4(df_mul({v.x, v.y}, ib), df_mul({v.z, v.w}, ib));
          vj[i] = v;
        }
        dacc_fma(ap, r, v.x, v.y);
        dacc_fma(ap, m, v.z, v.w);
        y[i] = df4(r, m);
      }
    }
    {
      const dfl s = df_block_sum2<kCoopDfWarps>(dacc_val(ap), red);
      if (tid == 0) pa[b] = s;
    }
    grid.sync();
    // ---- C1: alpha; w' into w; dots with w' recomputed on the fly
    const dfl a = coop_fixed_sum_df(pa, B, red + 40);  // next sum (a dot) uses red
    if (b == 0 && tid == 0) alpha[j] = df_val(a);
    if (j + 1 >= K_cap) break;  // identical in every block
    const dfl na = {-a.hi, -a.lo}, nb = {-bprev.hi, -bprev.lo};
    {
      dacc nw = {0.f, 0.f};
      for (int64_t i = gtid; i < n; i += gthreads) {
        const float4 x = three_term(y[i], vj[i], vjm1 ? vjm1 + i : nullptr, na, nb);
        w[i] = x;
        dacc_fma(nw, {x.x, x.y}, x.x, x.y);
        dacc_fma(nw, {x.z, x.w}, x.z, x.w);
      }
      const dfl s = df_block_sum2<kCoopDfWarps>(dacc_val(nw), red);  // |w'|^2 partial
      if (tid == 0) pw[b] = s;
    }
    const int m = j + 1;
    for (int k = b; k < m; k += B) {
      const float4* vk = V + (int64_t)k * n;
      dacc hr = {0.f, 0.f}, hm = {0.f, 0.f};
      int64_t i = tid;
      for (; i + kCoopDfThreads < n; i += 2 * kCoopDfThreads) {
        const int64_t i2 = i + kCoopDfThreads;
        const float4 a1 = vk[i], a2 = vk[i2];
        const float4 w1 = three_term(y[i], vj[i], vjm1 ? vjm1 + i : nullptr, na, nb);
        const float4 w2 = three_term(y[i2], vj[i2], vjm1 ? vjm1 + i2 : nullptr, na, nb);
        dot_acc(hr, hm, a1, w1);
        dot_acc(hr, hm, a2, w2);
      }
      if (i < n) dot_acc(hr, hm, vk[i], three_term(y[i], vj[i], vjm1 ? vjm1 + i : nullptr, na, nb));
      const dfl sr = df_block_sum2<kCoopDfWarps>(dacc_val(hr), red + 40);
      const dfl si = df_block_sum2<kCoopDfWarps>(dacc_val(hm), red);
      if (tid == 0) hc[k] = df4(sr, si);
    }
    grid.sync();
    // ---- D1, with the partials of |w|^2 after the first pass
    {
      const dfl s = project(m, true);
      if (tid == 0) pn[b] = s;
    }
    grid.sync();
    const dfl nw1 = coop_fixed_sum_df(pw, B, red + 40);
    dfl nw2 = coop_fixed_sum_df(pn, B, red);
    if (!(nw2.hi < 0.5f * nw1.hi)) {  // one pass was enough (identical in every block)
      const dfl bt = df_sqrt(nw2);
      if (b == 0 && tid == 0) {
        const double bd = df_val(bt);
        beta[j] = bd;
        if (!(bd > 0.0)) atomicExch(status, (int32_t)(bd == 0.0 ? EDGPU_ERR_BREAKDOWN : EDGPU_ERR_NAN));
      }
      __syncthreads();  // the next step's first sum reuses the buffer of nw2
      if (!(bt.hi > 0.f)) break;
      bprev = bt;
      continue;
    }
    // ---- C2
    for (int k = b; k < m; k += B) {
      const float4* vk = V + (int64_t)k * n;
      dacc hr = {0.f, 0.f}, hm = {0.f, 0.f};
      int64_t i = tid;
      for (; i + kCoopDfThreads < n; i += 2 * kCoopDfThreads) {
        const int64_t i2 = i + kCoopDfThreads;
        const float4 a1 = vk[i], a2 = vk[i2], x1 = w[i], x2 = w[i2];
        dot_acc(hr, hm, a1, x1);
        dot_acc(hr, hm, a2, x2);
      }
      if (i < n) dot_acc(hr, hm, vk[i], w[i]);
      const dfl sr = df_block_sum2<kCoopDfWarps>(dacc_val(hr), red + 40);
      const dfl si = df_block_sum2<kCoopDfWarps>(dacc_val(hm), red);
      if (tid == 0) hc[k] = df4(sr, si);
    }
    grid.sync();
    // ---- D2 and beta_j
    {
      const dfl s = project(m, true);
      if (tid == 0) pn[b] = s;
    }
    grid.sync();
    const dfl bt = df_sqrt(coop_fixed_sum_df(pn, B, red + 40));  // next sum (alpha partials) uses red
    if (b == 0 && tid == 0) {
      const double bd = df_val(bt);
      beta[j] = bd;
      if (!(bd > 0.0)) atomicExch(status, (int32_t)(bd == 0.0 ? EDGPU_ERR_BREAKDOWN : EDGPU_ERR_NAN));
    }
    if (!(bt.hi > 0.f)) break;  // identical in every block
    bprev = bt;
  }
}

}  // namespace edgpu

using namespace edgpu;

extern "C" int edgpu_lanczos_reorth_df(const edgpu_csr* h, const double* v0, int j0, int j1, int K_cap, double* Vd,
                                       double* wd, double* alpha, double* beta, int32_t* status_dev, void* workspace,
                                       size_t workspace_bytes, void* stream) {
  if (!h || !Vd || !wd || !alpha || !beta || !status_dev || h->n < 1) return EDGPU_ERR_ARG;
  if (j0 < 0 || j1 > K_cap || j0 > j1) return EDGPU_ERR_ARG;
  if (j0 == 0 && !v0) return EDGPU_ERR_ARG;
  if (!h->val_df || h->val_c || h->n > kCoopDfMaxN) return EDGPU_ERR_ARG;
  const int64_t n = h->n;
  const size_t need = sizeof(float4) * (size_t)n + 3 * sizeof(dfl) * kCoopDfMaxBlocks +
                      sizeof(float4) * (size_t)(K_cap + 1) + 4 * 256;
  if (workspace_bytes < need) return EDGPU_ERR_WORKSPACE;
  if (j0 == j1) return EDGPU_OK;
  int dev = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
      !coop) {
    cudaGetLastError();
    return EDGPU_ERR_ARG;
  }
  int per_sm = 0;
  if (cudaFuncSetAttribute(lanczos_reorth_coop_df_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)kCacheBytes) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lanczos_reorth_coop_df_kernel, kCoopDfThreads,
                                                    kCacheBytes) != cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    return EDGPU_ERR_ARG;
  }
  int blocks = grid_cap();  // one block per SM
  if (blocks > kCoopDfMaxBlocks) blocks = kCoopDfMaxBlocks;
  unsigned char* ws = reinterpret_cast<unsigned char*>(workspace);
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    unsigned char* p = ws + off;
    off += (bytes + 255) & ~(size_t)255;
    return p;
  };
  float4* y = reinterpret_cast<float4*>(carve(sizeof(float4) * (size_t)n));
  dfl* pa = reinterpret_cast<dfl*>(carve(sizeof(dfl) * kCoopDfMaxBlocks));
  dfl* pn = reinterpret_cast<dfl*>(carve(sizeof(dfl) * kCoopDfMaxBlocks));
  dfl* pw = reinterpret_cast<dfl*>(carve(sizeof(dfl) * kCoopDfMaxBlocks));
  float4* hc = reinterpret_cast<float4*>(carve(sizeof(float4) * (size_t)(K_cap + 1)));
  const int64_t* rp = h->row_ptr;
  const int32_t* col = h->col;
  const float2* hv = reinterpret_cast<const float2*>(h->val_df);
  const double2* v0c = reinterpret_cast<const double2*>(v0);
  float4* V = reinterpret_cast<float4*>(Vd);
  float4* w = reinterpret_cast<float4*>(wd);
  void* args[] = {(void*)&n, (void*)&rp, (void*)&col, (void*)&hv, (void*)&v0c, (void*)&j0, (void*)&j1, (void*)&K_cap,
                  (void*)&V, (void*)&w, (void*)&y, (void*)&alpha, (void*)&beta, (void*)&status_dev, (void*)&pa,
                  (void*)&pn, (void*)&pw, (void*)&hc};
  const cudaError_t e = cudaLaunchCooperativeKernel((const void*)lanczos_reorth_coop_df_kernel, blocks, kCoopDfThreads,
                                                    args, kCacheBytes, (cudaStream_t)stream);
  note_launch();
  if (e != cudaSuccess) {
    cudaGetLastError();
    return EDGPU_ERR_CUDA;
  }
  return check_launch();
}
