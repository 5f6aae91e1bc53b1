// Connected components of a sector's Hamiltonian graph, labelled by their smallest member.
//
// The Krylov size of each Green's-function run is upstream's min(krylovSize, dimension of the
// run's own basis closure) (impurityModel/ed/spectra.py:646-676 with the expand_basis of
// finite.py:1696-1803); on the shared sector of a batch that dimension is the size of the
// connected components the run's start states touch.  For sectors up to kCcMaxRows states one
// CTA iterates minimum-label propagation with pointer jumping on chip until nothing changes
// (at most n + 1 rounds, each bounded), so the host reads the labels once instead of
// synchronising on every round.
#include "common.cuh"

namespace edgpu {

constexpr int kCcThreads = 1024;
constexpr int64_t kCcMaxRows = 1 << 16;

__global__ void __launch_bounds__(kCcThreads)
    components_kernel(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                      int64_t* __restrict__ label, int32_t* __restrict__ rounds_out) {
  __shared__ int changed;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) label[i] = i;
  __syncthreads();
  int rounds = 0;
  for (int64_t it = 0; it <= n; ++it) {
    if (threadIdx.x == 0) changed = 0;
    __syncthreads();
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      int64_t m = label[i];
      const int64_t e1 = rp[i + 1];
      for (int64_t e = rp[i]; e < e1; ++e) {
        const int64_t lj = label[col[e]];
        m = lj < m ? lj : m;
      }
      const int64_t jm = label[m];  // pointer jumping
      m = jm < m ? jm : m;
      if (m < label[i]) {
        atomicMin(reinterpret_cast<unsigned long long*>(label + i), (unsigned long long)m);
        changed = 1;
      }
    }
    __syncthreads();
    ++rounds;
    const int c = changed;
    __syncthreads();
    if (!c) break;
  }
  if (threadIdx.x == 0 && rounds_out) *rounds_out = rounds;
}

}  // namespace edgpu

using namespace edgpu;

extern "C" int edgpu_components(const edgpu_csr* h, int64_t* label, int32_t* rounds, void* stream) {
  if (!h || !label || h->n < 0) return EDGPU_ERR_ARG;
  if (h->n == 0) return EDGPU_OK;
  if (h->n > kCcMaxRows || (h->nnz > 0 && (!h->row_ptr || !h->col))) return EDGPU_ERR_ARG;
  components_kernel<<<1, kCcThreads, 0, (cudaStream_t)stream>>>(h->n, h->row_ptr, h->col, label, rounds);
  note_launch();
  return check_launch();
}
