// One-body density matrices of many states at once.
//
// Replaces upstream's per-entry loops over dict states (impurityModel/ed/finite.py:967-1012,
// getDensityMatrix: a(i), c(j), inner product per (i, j) pair; and the occupation sums of
// getTraceDensityMatrix / getLz3d / getSz3d / getEgT2gOccupation, finite.py:843-1112, which
// are linear functions of the same matrix).  One block per (pair, state): every thread takes
// product states of the state's sorted support, applies c_j^dagger c_i with upstream's sign
// rule, finds the target in the sorted support by binary search and accumulates
// conj(a_target) * sign * a_source; a fixed-order block reduction gives the entry.
#include "common.cuh"

namespace edgpu {

constexpr int kDmThreads = 256;

template <int W>
__global__ void __launch_bounds__(kDmThreads)
    density_matrix_kernel(const uint64_t* __restrict__ states, const double2* __restrict__ amps,
                          const int64_t* __restrict__ run_off, int R, const uint64_t* __restrict__ pair_ops, int P,
                          double2* __restrict__ out) {
  __shared__ double red_r[kDmThreads / 32], red_i[kDmThreads / 32];
  const int p = blockIdx.x, r = blockIdx.y;
  if (p >= P || r >= R) return;
  const int64_t a0 = run_off[r], a1 = run_off[r + 1];
  const uint64_t* base = states + a0 * W;
  const int64_t n = a1 - a0;
  const uint64_t ops = pair_ops[p];
  double re = 0.0, im = 0.0;
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
    uint64_t s[W];
    load_state<W>(base + k * W, s);
    int parity = 0;
    if (!apply_term<W>(s, ops, parity)) continue;
    const int64_t q = find_state<W>(base, n, s);
    if (q < 0) continue;
    const double2 ak = amps[a0 + k], aq = amps[a0 + q];
    const double sg = (parity & 1) ? -1.0 : 1.0;
    re += sg * (aq.x * ak.x + aq.y * ak.y);
    im += sg * (aq.x * ak.y - aq.y * ak.x);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_down_sync(0xffffffffu, re, o);
    im += __shfl_down_sync(0xffffffffu, im, o);
  }
  if (lane == 0) {
    red_r[warp] = re;
    red_i[warp] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sr = 0.0, si = 0.0;
    for (int q = 0; q < kDmThreads / 32; ++q) {
      sr += red_r[q];
      si += red_i[q];
    }
    out[(int64_t)r * P + p] = make_double2(sr, si);
  }
}

}  // namespace edgpu

using namespace edgpu;

extern "C" int edgpu_density_matrix(int n_words, const uint64_t* states, const double* amps, const int64_t* run_off,
                                    int R, const uint64_t* pair_ops, int P, double* out, void* stream) {
  if (R < 0 || P < 0 || (R > 0 && P > 0 && (!states || !amps || !run_off || !pair_ops || !out)))
    return EDGPU_ERR_ARG;
  if (R == 0 || P == 0) return EDGPU_OK;
  if (R > 65535) return EDGPU_ERR_ARG;
  dim3 grid(P, R);
  EDGPU_DISPATCH_W(n_words, {
    density_matrix_kernel<W><<<grid, kDmThreads, 0, (cudaStream_t)stream>>>(
        states, reinterpret_cast<const double2*>(amps), run_off, R, pair_ops, P, reinterpret_cast<double2*>(out));
    note_launch();
  });
  return check_launch();
}
