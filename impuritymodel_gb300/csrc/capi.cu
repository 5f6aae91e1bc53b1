// Version and status strings of the edgpu C ABI.
#include <atomic>

#include "common.cuh"

namespace edgpu {
static std::atomic<long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
}  // namespace edgpu

extern "C" long long edgpu_launch_count(void) { return edgpu::g_launches.load(std::memory_order_relaxed); }

extern "C" int edgpu_abi_version(void) { return EDGPU_ABI_VERSION; }

extern "C" const char* edgpu_status_string(int status) {
  switch (status) {
    case EDGPU_OK: return "ok";
    case EDGPU_ERR_ARG: return "bad argument";
    case EDGPU_ERR_OVERFLOW: return "scratch or output capacity exceeded";
    case EDGPU_ERR_BREAKDOWN: return "Lanczos breakdown (beta == 0)";
    case EDGPU_ERR_NAN: return "non-finite value";
    case EDGPU_ERR_NOCONV: return "not converged within the iteration cap";
    case EDGPU_ERR_CUDA: return "CUDA error";
    case EDGPU_ERR_WORKSPACE: return "workspace too small";
    default: return "unknown status";
  }
}
