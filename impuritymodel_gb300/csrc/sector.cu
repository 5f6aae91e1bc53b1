// Single-call sector construction and ground state for hosts without the Python layer
// (edgpu_build_csr, edgpu_expand, edgpu_eig_lowest).  Each is host orchestration in C++ over
// the library's own kernels (operator application, scan, sort, unique, merge, reorthogonalised
// Lanczos, combination), synchronous on the caller's stream (sizes are read back between
// phases), with all scratch carved from the caller's workspace.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace edgpu {
namespace {

// Bump allocator over the caller's workspace (256-byte aligned pieces).
struct Arena {
  unsigned char* base;
  size_t size, off = 0;
  bool ok = true;
  template <typename T>
  T* take(size_t count) {
    const size_t bytes = (sizeof(T) * count + 255) & ~(size_t)255;
    if (off + bytes > size) {
      ok = false;
      return nullptr;
    }
    T* p = reinterpret_cast<T*>(base + off);
    off += bytes;
    return p;
  }
};

inline size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

template <typename T>
int d2h(T* dst, const T* src, size_t count, cudaStream_t s) {
  if (cudaMemcpyAsync(dst, src, sizeof(T) * count, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return EDGPU_ERR_CUDA;
  return EDGPU_OK;
}

__global__ void index_to_col_kernel(const int64_t* __restrict__ idx, int64_t m, int32_t* col) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) col[i] = (int32_t)idx[i];
}

__global__ void real_part_kernel(const double2* __restrict__ v, int64_t m, double* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) out[i] = v[i].x;
}

__global__ void iota_u32_kernel(uint32_t* p, int64_t m) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) p[i] = (uint32_t)i;
}

inline unsigned blocks_for(int64_t m) { return (unsigned)((m + 255) / 256); }

// Per-state count pass of edgpu_apply_columns with the scratch capacity grown on overflow
// (as the Python engine does); counts[n], the scan into offsets[n + 1]; *total on the host.
int count_and_scan(int w, const uint64_t* states, int64_t n, const edgpu_terms* terms, const edgpu_restrictions* restr,
                   double weight_min, const uint64_t* basis, int64_t nb, int filter, int64_t* counts,
                   int64_t* offsets, void* scan_ws, size_t scan_bytes, int* scratch, int32_t* status,
                   int64_t* total, cudaStream_t s) {
  for (;;) {
    if (cudaMemsetAsync(status, 0, sizeof(int32_t), s) != cudaSuccess) return EDGPU_ERR_CUDA;
    int rc = edgpu_apply_columns(w, states, n, terms, restr, weight_min, basis, nb, filter, nullptr, counts, nullptr,
                                 nullptr, nullptr, 0, *scratch, status, s);
    if (rc) return rc;
    if ((rc = edgpu_scan_i64(counts, offsets, n, scan_ws, scan_bytes, s))) return rc;
    int32_t st = 0;
    if ((rc = d2h(&st, status, 1, s))) return rc;
    if (st == EDGPU_ERR_OVERFLOW && *scratch < 8192) {
      *scratch *= 4;
      continue;
    }
    if (st) return st;
    return d2h(total, offsets + n, 1, s);
  }
}

// Sorted unique copy of keys[m] (in place: keys sorted, first u rows unique) -> *u.
int sort_unique_inplace(int w, uint64_t* keys, int64_t m, uint64_t* tmp_keys, uint32_t* payload, int64_t* head,
                        int64_t* hscan, uint32_t* first, void* sort_ws, size_t sort_bytes, void* scan_ws,
                        size_t scan_bytes, int64_t* u, cudaStream_t s) {
  if (m == 0) {
    *u = 0;
    return EDGPU_OK;
  }
  iota_u32_kernel<<<blocks_for(m), 256, 0, s>>>(payload, m);
  note_launch();
  int rc = edgpu_sort_states(w, keys, payload, m, nullptr, sort_ws, sort_bytes, s);
  if (rc) return rc;
  if ((rc = edgpu_segment_heads(w, keys, m, head, s))) return rc;
  if ((rc = edgpu_scan_i64(head, hscan, m, scan_ws, scan_bytes, s))) return rc;
  if ((rc = edgpu_segment_reduce(w, keys, payload, m, hscan, nullptr, tmp_keys, first, nullptr, s))) return rc;
  if ((rc = d2h(u, hscan + m, 1, s))) return rc;
  if (cudaMemcpyAsync(keys, tmp_keys, sizeof(uint64_t) * (size_t)w * (size_t)*u, cudaMemcpyDeviceToDevice, s) !=
      cudaSuccess)
    return EDGPU_ERR_CUDA;
  return check_launch();
}

// ---------------------------------------------------------------------------------------
// Lowest eigenpairs of a symmetric tridiagonal matrix (diagonal a[m], off-diagonal b[m-1]):
// eigenvalues by bisection on Sturm sequence counts, eigenvectors by inverse iteration with
// partial-pivoting LU of the shifted tridiagonal, orthogonalised within clusters.
// ---------------------------------------------------------------------------------------
int sturm_count(const std::vector<double>& a, const std::vector<double>& b, double x) {
  // number of eigenvalues below x (LDL^T pivots of T - x I that are negative)
  int c = 0;
  double d = a[0] - x;
  const double tiny = 1e-300;
  if (d < 0) ++c;
  for (size_t i = 1; i < a.size(); ++i) {
    if (std::fabs(d) < tiny) d = -tiny;
    d = (a[i] - x) - b[i - 1] * b[i - 1] / d;
    if (d < 0) ++c;
  }
  return c;
}

void tridiag_lowest(const std::vector<double>& a, const std::vector<double>& b, int q, std::vector<double>& th,
                    std::vector<std::vector<double>>& vec) {
  const int m = (int)a.size();
  double lo = a[0], hi = a[0];
  for (int i = 0; i < m; ++i) {
    const double r = (i > 0 ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < m ? std::fabs(b[i]) : 0.0);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
  }
  const double span = std::max(hi - lo, 1e-300);
  th.assign(q, 0.0);
  for (int k = 0; k < q; ++k) {
    // the (k+1)-th smallest: largest x with count(x) <= k
    double l = lo - 1e-12 * span, h = hi + 1e-12 * span;
    for (int it = 0; it < 200 && h - l > 4e-16 * std::max(std::fabs(l), std::fabs(h)) + 1e-300; ++it) {
      const double mid = 0.5 * (l + h);
      if (sturm_count(a, b, mid) <= k)
        l = mid;
      else
        h = mid;
    }
    th[k] = 0.5 * (l + h);
  }
  vec.assign(q, std::vector<double>(m, 0.0));
  std::vector<double> d(m), du(m, 0.0), du2(m, 0.0), l(m, 0.0);
  std::vector<char> sw(m, 0);
  for (int k = 0; k < q; ++k) {
    // LU with partial pivoting of T - shift I (rows swapped where the sub-diagonal entry is
    // the larger pivot; U gets a second super-diagonal where rows were swapped)
    const double shift = th[k] + 1e-14 * span * (k % 2 ? 1.0 : -1.0);
    for (int i = 0; i < m; ++i) {
      d[i] = a[i] - shift;
      du[i] = i + 1 < m ? b[i] : 0.0;
      du2[i] = 0.0;
      sw[i] = 0;
    }
    for (int i = 0; i + 1 < m; ++i) {
      const double sub = b[i];
      if (std::fabs(d[i]) >= std::fabs(sub)) {
        const double f = d[i] != 0.0 ? sub / d[i] : 0.0;
        l[i] = f;
        d[i + 1] -= f * du[i];
      } else {
        const double f = d[i] / sub;
        const double d1 = d[i + 1], u0 = du[i];
        sw[i] = 1;
        l[i] = f;
        d[i] = sub;
        du[i] = d1;
        d[i + 1] = u0 - f * d1;
        if (i + 2 < m) {
          du2[i] = du[i + 1];
          du[i + 1] = -f * du[i + 1];
        }
      }
    }
    for (int i = 0; i < m; ++i)
      if (std::fabs(d[i]) < 1e-300) d[i] = 1e-300;
    std::vector<double>& x = vec[k];
    for (int i = 0; i < m; ++i) x[i] = (1.0 + 0.01 * std::sin(1.0 + i + 7.0 * k)) / std::sqrt((double)m);
    for (int it = 0; it < 3; ++it) {
      std::vector<double> y(x);
      for (int i = 0; i + 1 < m; ++i) {
        if (sw[i]) std::swap(y[i], y[i + 1]);
        y[i + 1] -= l[i] * y[i];
      }
      for (int i = m - 1; i >= 0; --i) {
        double v = y[i];
        if (i + 1 < m) v -= du[i] * y[i + 1];
        if (i + 2 < m) v -= du2[i] * y[i + 2];
        y[i] = v / d[i];
      }
      // orthogonal to the earlier vectors of the same cluster
      for (int j = 0; j < k; ++j)
        if (std::fabs(th[j] - th[k]) < 1e-8 * span) {
          double dot = 0.0;
          for (int i = 0; i < m; ++i) dot += vec[j][i] * y[i];
          for (int i = 0; i < m; ++i) y[i] -= dot * vec[j][i];
        }
      double nrm = 0.0;
      for (int i = 0; i < m; ++i) nrm += y[i] * y[i];
      nrm = std::sqrt(nrm);
      for (int i = 0; i < m; ++i) x[i] = y[i] / nrm;
    }
  }
}

// v[i] = complex normal numbers from a counter-based generator (splitmix64 + Box-Muller)
__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void random_start_kernel(int64_t n, uint64_t seed, double2* v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t a = splitmix64(seed ^ (2 * (uint64_t)i)), b = splitmix64(seed ^ (2 * (uint64_t)i + 1));
  const double u1 = ((a >> 11) + 1.0) * (1.0 / 9007199254740993.0), u2 = (b >> 11) * (1.0 / 9007199254740992.0);
  const double r = sqrt(-2.0 * log(u1));
  double sn, cs;
  sincospi(2.0 * u2, &sn, &cs);
  v[i] = make_double2(r * cs, r * sn);
}

__global__ void scale_kernel(double2* v, int64_t n, const double* nrm2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double f = 1.0 / sqrt(*nrm2);
  v[i].x *= f;
  v[i].y *= f;
}

__global__ void norm2_kernel(const double2* __restrict__ v, int64_t n, double* out) {
  // one block, fixed order
  __shared__ double red[1024];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += v[i].x * v[i].x + v[i].y * v[i].y;
  red[threadIdx.x] = s;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

}  // namespace
}  // namespace edgpu

using namespace edgpu;

// ---------------------------------------------------------------------------------------
extern "C" size_t edgpu_build_csr_workspace(int n_words, int64_t n, int64_t nnz_cap) {
  if (n < 1 || n_words < 1 || n_words > EDGPU_MAX_WORDS || nnz_cap < 0) return 0;
  return 1024 + al(8 * (size_t)n) + al(edgpu_scan_workspace(n)) + al(8 * (size_t)nnz_cap) +
         al(16 * (size_t)nnz_cap);
}

extern "C" int edgpu_build_csr(int n_words, const edgpu_terms* terms, const edgpu_restrictions* restr,
                               double weight_min, const uint64_t* basis, int64_t n, int real_values, int64_t* row_ptr,
                               int32_t* col, double* val, int64_t nnz_cap, int64_t* nnz_out, int32_t* status_dev,
                               void* workspace, size_t workspace_bytes, void* stream) {
  if (!terms || !basis || n < 1 || !row_ptr || !nnz_out || !status_dev || nnz_cap < 0) return EDGPU_ERR_ARG;
  if (n_words < 1 || n_words > EDGPU_MAX_WORDS) return EDGPU_ERR_ARG;
  if (workspace_bytes < edgpu_build_csr_workspace(n_words, n, nnz_cap)) return EDGPU_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  Arena ar{reinterpret_cast<unsigned char*>(workspace), workspace_bytes};
  int64_t* counts = ar.take<int64_t>(n);
  unsigned char* scan_ws = ar.take<unsigned char>(edgpu_scan_workspace(n));
  int64_t* idx = ar.take<int64_t>(nnz_cap > 0 ? nnz_cap : 1);
  double2* vals = ar.take<double2>(nnz_cap > 0 ? nnz_cap : 1);
  if (!ar.ok) return EDGPU_ERR_WORKSPACE;
  int scratch = 256;
  int64_t total = 0;
  int rc = count_and_scan(n_words, basis, n, terms, restr, weight_min, basis, n, EDGPU_FILTER_IN_BASIS, counts,
                          row_ptr, scan_ws, edgpu_scan_workspace(n), &scratch, status_dev, &total, s);
  if (rc) return rc;
  *nnz_out = total;
  if (total > nnz_cap || (total > 0 && (!col || !val))) return EDGPU_ERR_OVERFLOW;
  if (total == 0) return EDGPU_OK;
  if (cudaMemsetAsync(status_dev, 0, sizeof(int32_t), s) != cudaSuccess) return EDGPU_ERR_CUDA;
  // row j holds H|b_j> conjugated: row j of the Hermitian H
  double2* vout = real_values ? vals : reinterpret_cast<double2*>(val);
  rc = edgpu_apply_columns(n_words, basis, n, terms, restr, weight_min, basis, n, EDGPU_FILTER_IN_BASIS, row_ptr,
                           nullptr, nullptr, idx, reinterpret_cast<double*>(vout), 1, scratch, status_dev, s);
  if (rc) return rc;
  index_to_col_kernel<<<blocks_for(total), 256, 0, s>>>(idx, total, col);
  note_launch();
  if (real_values) {
    real_part_kernel<<<blocks_for(total), 256, 0, s>>>(vals, total, val);
    note_launch();
  }
  int32_t st = 0;
  if ((rc = d2h(&st, status_dev, 1, s))) return rc;
  return st ? st : check_launch();
}

// ---------------------------------------------------------------------------------------
extern "C" size_t edgpu_expand_workspace(int n_words, int64_t capacity, int64_t emit_cap) {
  if (n_words < 1 || n_words > EDGPU_MAX_WORDS || capacity < 1 || emit_cap < 1) return 0;
  const int64_t big = std::max(capacity, emit_cap) * 2;
  const size_t W8 = 8 * (size_t)n_words;
  return 4096 + al(edgpu_sort_states_workspace(n_words, big)) + al(edgpu_scan_workspace(big)) +
         4 * al(W8 * (size_t)capacity) + 2 * al(W8 * (size_t)big) + 3 * al(8 * (size_t)big) +
         2 * al(4 * (size_t)big) + 2 * al(8 * (size_t)(capacity + 1));
}

extern "C" int edgpu_expand(int n_words, const edgpu_terms* terms, const edgpu_restrictions* restr,
                            double weight_min, const uint64_t* basis0, int64_t n0, int64_t capacity,
                            int64_t emit_cap, uint64_t* out_sorted, uint64_t* out_layered, int64_t* n_out,
                            int32_t* status_dev, void* workspace, size_t workspace_bytes, void* stream) {
  if (!terms || !basis0 || n0 < 1 || !out_sorted || !n_out || !status_dev || capacity < n0 || emit_cap < 1)
    return EDGPU_ERR_ARG;
  if (n_words < 1 || n_words > EDGPU_MAX_WORDS) return EDGPU_ERR_ARG;
  if (workspace_bytes < edgpu_expand_workspace(n_words, capacity, emit_cap)) return EDGPU_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const int w = n_words;
  const size_t W8 = 8 * (size_t)w;
  const int64_t big = std::max(capacity, emit_cap) * 2;
  Arena ar{reinterpret_cast<unsigned char*>(workspace), workspace_bytes};
  unsigned char* sort_ws = ar.take<unsigned char>(edgpu_sort_states_workspace(w, big));
  unsigned char* scan_ws = ar.take<unsigned char>(edgpu_scan_workspace(big));
  uint64_t* frontier = ar.take<uint64_t>((size_t)w * capacity);
  uint64_t* layer = ar.take<uint64_t>((size_t)w * capacity);
  uint64_t* merged = ar.take<uint64_t>((size_t)w * capacity);
  uint64_t* spare = ar.take<uint64_t>((size_t)w * capacity);
  uint64_t* cand = ar.take<uint64_t>((size_t)w * big);
  uint64_t* tmpk = ar.take<uint64_t>((size_t)w * big);
  int64_t* counts = ar.take<int64_t>(big);
  int64_t* offsets = ar.take<int64_t>(big + 1);
  int64_t* head = ar.take<int64_t>(big);
  uint32_t* payload = ar.take<uint32_t>(big);
  uint32_t* first = ar.take<uint32_t>(big);
  int64_t* hscan = ar.take<int64_t>(big + 1);
  if (!ar.ok) return EDGPU_ERR_WORKSPACE;
  (void)spare;
  const size_t sort_bytes = edgpu_sort_states_workspace(w, big), scan_bytes = edgpu_scan_workspace(big);
  int rc;
  // sorted unique copy of basis0; the layered order starts with basis0 as given
  if (cudaMemcpyAsync(cand, basis0, W8 * (size_t)n0, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return EDGPU_ERR_CUDA;
  int64_t ns = 0;
  if ((rc = sort_unique_inplace(w, cand, n0, tmpk, payload, head, hscan, first, sort_ws, sort_bytes, scan_ws,
                                scan_bytes, &ns, s)))
    return rc;
  if (cudaMemcpyAsync(out_sorted, cand, W8 * (size_t)ns, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(frontier, basis0, W8 * (size_t)n0, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return EDGPU_ERR_CUDA;
  int64_t nl = 0;
  if (out_layered) {
    if (cudaMemcpyAsync(out_layered, basis0, W8 * (size_t)n0, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return EDGPU_ERR_CUDA;
    nl = n0;
  }
  int64_t nf = n0;
  int scratch = 256;
  std::vector<int64_t> off_h;
  while (nf > 0) {
    // candidates of the frontier not yet in the basis, in chunks of at most emit_cap
    int64_t total = 0;
    if ((rc = count_and_scan(w, frontier, nf, terms, restr, weight_min, out_sorted, ns, EDGPU_FILTER_NOT_IN_BASIS,
                             counts, offsets, scan_ws, scan_bytes, &scratch, status_dev, &total, s)))
      return rc;
    if (total == 0) break;
    off_h.resize((size_t)nf + 1);
    if ((rc = d2h(off_h.data(), offsets, (size_t)nf + 1, s))) return rc;
    int64_t nlayer = 0;  // sorted unique new states of this layer so far (in `layer`)
    int64_t a = 0;
    while (a < nf) {
      int64_t b = a + 1;
      while (b < nf && off_h[b + 1] - off_h[a] <= emit_cap) ++b;
      const int64_t ca = off_h[b] - off_h[a];
      if (ca > emit_cap) return EDGPU_ERR_OVERFLOW;  // one state emits more than emit_cap
      if (ca > 0) {
        int64_t sub_total = 0;
        if ((rc = count_and_scan(w, frontier + (size_t)a * w, b - a, terms, restr, weight_min, out_sorted, ns,
                                 EDGPU_FILTER_NOT_IN_BASIS, counts, offsets, scan_ws, scan_bytes, &scratch,
                                 status_dev, &sub_total, s)))
          return rc;
        if (cudaMemsetAsync(status_dev, 0, sizeof(int32_t), s) != cudaSuccess) return EDGPU_ERR_CUDA;
        if ((rc = edgpu_apply_columns(w, frontier + (size_t)a * w, b - a, terms, restr, weight_min, out_sorted, ns,
                                      EDGPU_FILTER_NOT_IN_BASIS, offsets, nullptr, cand + (size_t)nlayer * w,
                                      nullptr, nullptr, 0, scratch, status_dev, s)))
          return rc;
        // cand = [layer so far | this chunk]: sort, unique
        if (nlayer > 0 &&
            cudaMemcpyAsync(cand, layer, W8 * (size_t)nlayer, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
          return EDGPU_ERR_CUDA;
        int64_t u = 0;
        if ((rc = sort_unique_inplace(w, cand, nlayer + sub_total, tmpk, payload, head, hscan, first, sort_ws,
                                      sort_bytes, scan_ws, scan_bytes, &u, s)))
          return rc;
        if (ns + u > capacity) {
          *n_out = ns + u;
          return EDGPU_ERR_OVERFLOW;
        }
        if (cudaMemcpyAsync(layer, cand, W8 * (size_t)u, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
          return EDGPU_ERR_CUDA;
        nlayer = u;
      }
      a = b;
    }
    if (nlayer == 0) break;
    if ((rc = edgpu_merge_states(w, out_sorted, ns, layer, nlayer, merged, s))) return rc;
    if (cudaMemcpyAsync(out_sorted, merged, W8 * (size_t)(ns + nlayer), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return EDGPU_ERR_CUDA;
    ns += nlayer;
    if (out_layered) {
      if (cudaMemcpyAsync(out_layered + (size_t)nl * w, layer, W8 * (size_t)nlayer, cudaMemcpyDeviceToDevice, s) !=
          cudaSuccess)
        return EDGPU_ERR_CUDA;
      nl += nlayer;
    }
    if (cudaMemcpyAsync(frontier, layer, W8 * (size_t)nlayer, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return EDGPU_ERR_CUDA;
    nf = nlayer;
  }
  *n_out = ns;
  if (cudaStreamSynchronize(s) != cudaSuccess) return EDGPU_ERR_CUDA;
  return check_launch();
}

// ---------------------------------------------------------------------------------------
extern "C" size_t edgpu_eig_lowest_workspace(int64_t n, int k_cap) {
  if (n < 1 || k_cap < 1) return 0;
  return 4096 + al(16 * (size_t)n * (size_t)k_cap) + 2 * al(16 * (size_t)n) + 4 * al(8 * (size_t)(k_cap + 1)) +
         al(16 * (size_t)k_cap * (size_t)k_cap) + al(edgpu_lanczos_reorth_workspace(n, k_cap));
}

extern "C" int edgpu_eig_lowest(const edgpu_csr* h, int k, double tol_rel, int k_cap, uint64_t seed, double* evals,
                                double* evecs, int* k_found, int32_t* status_dev, void* workspace,
                                size_t workspace_bytes, void* stream) {
  if (!h || h->n < 1 || k < 1 || k_cap < 1 || !evals || !evecs || !k_found || !status_dev || !(tol_rel > 0))
    return EDGPU_ERR_ARG;
  const int64_t n = h->n;
  if (k_cap > n) k_cap = (int)n;
  if (k > k_cap) return EDGPU_ERR_ARG;
  if (workspace_bytes < edgpu_eig_lowest_workspace(n, k_cap)) return EDGPU_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  Arena ar{reinterpret_cast<unsigned char*>(workspace), workspace_bytes};
  double2* V = ar.take<double2>((size_t)n * k_cap);
  double2* v0 = ar.take<double2>(n);
  double2* wv = ar.take<double2>(n);
  double* alpha = ar.take<double>(k_cap + 1);
  double* beta = ar.take<double>(k_cap + 1);
  double* nrm = ar.take<double>(2);
  double2* coef = ar.take<double2>((size_t)k_cap * k_cap);
  unsigned char* lws = ar.take<unsigned char>(edgpu_lanczos_reorth_workspace(n, k_cap));
  if (!ar.ok) return EDGPU_ERR_WORKSPACE;
  random_start_kernel<<<blocks_for(n), 256, 0, s>>>(n, seed, v0);
  norm2_kernel<<<1, 1024, 0, s>>>(v0, n, nrm);
  scale_kernel<<<blocks_for(n), 256, 0, s>>>(v0, n, nrm);
  note_launch();
  note_launch();
  note_launch();
  if (cudaMemsetAsync(status_dev, 0, sizeof(int32_t), s) != cudaSuccess) return EDGPU_ERR_CUDA;
  std::vector<double> ah, bh;
  std::vector<double> th;
  std::vector<std::vector<double>> sv;
  int j = 0, done = 0;
  const int chunk = 32;
  int rc;
  while (!done) {
    const int j1 = std::min(k_cap, j + chunk);
    rc = edgpu_lanczos_reorth(h, reinterpret_cast<const double*>(v0), j, j1, k_cap, reinterpret_cast<double*>(V),
                              reinterpret_cast<double*>(wv), alpha, beta, status_dev, lws,
                              edgpu_lanczos_reorth_workspace(n, k_cap), s);
    if (rc) return rc;
    int32_t st = 0;
    if ((rc = d2h(&st, status_dev, 1, s))) return rc;
    ah.resize(j1);
    bh.resize(j1);
    if ((rc = d2h(ah.data(), alpha, j1, s)) || (rc = d2h(bh.data(), beta, j1, s))) return rc;
    int m = j1;
    bool exact = j1 >= n;
    if (st == EDGPU_ERR_BREAKDOWN) {
      for (m = 1; m <= j1 && bh[m - 1] != 0.0; ++m) {
      }
      m = std::min(m, j1);
      exact = true;
    } else if (st) {
      return st;
    }
    const int q = std::min(k, m);
    std::vector<double> a(ah.begin(), ah.begin() + m), b(bh.begin(), bh.begin() + (m > 1 ? m - 1 : 0));
    tridiag_lowest(a, b, q, th, sv);
    bool conv = q == k || exact;
    if (!exact)
      for (int i = 0; i < q && conv; ++i) {
        const double res = std::fabs(bh[m - 1] * sv[i][m - 1]);
        conv = res <= tol_rel * std::max(1.0, std::fabs(th[i]));
      }
    if (conv || exact || j1 >= k_cap) {
      // Ritz vectors X[i] = sum_l s[i][l] V[l]
      std::vector<double2> c((size_t)m * q);
      for (int l = 0; l < m; ++l)
        for (int i = 0; i < q; ++i) c[(size_t)l * q + i] = make_double2(sv[i][l], 0.0);
      if (cudaMemcpyAsync(coef, c.data(), sizeof(double2) * c.size(), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return EDGPU_ERR_CUDA;
      if ((rc = edgpu_combine(reinterpret_cast<const double*>(V), m, n, reinterpret_cast<const double*>(coef), q,
                              evecs, s)))
        return rc;
      for (int i = 0; i < q; ++i) evals[i] = th[i];
      *k_found = q;
      if (cudaStreamSynchronize(s) != cudaSuccess) return EDGPU_ERR_CUDA;
      if (!(conv || exact)) return EDGPU_ERR_NOCONV;
      done = 1;
    }
    j = j1;
  }
  return check_launch();
}
