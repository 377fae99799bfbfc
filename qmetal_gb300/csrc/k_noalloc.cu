// k_noalloc.cu -- the fused diagonal layer for callers that cannot allocate
// device memory.
//
// Some callers of this library may not call cudaMalloc: an application that
// hands all device memory to its own allocator or pool and forbids other
// allocations, a plugin whose host only lends it pointers and a stream, or a
// latency-critical loop where an allocation could synchronise the device.
// They still own the state; what they cannot provide is the scratch the
// diagonal layer needs (a term descriptor and the 2^13-entry low-bit phase
// table). This entry point runs the same kernels as qmk_apply_diagonal with
// that scratch in a file-scope device array, so the call allocates nothing.
//
// Scratch: one workspace of qmk_workspace_bytes() (the same for every n),
// 327 KiB per device that loads this library, held until the process exits.
// Every call shares it: the prep kernel rewrites the descriptor and the table
// before the pass reads them, so nothing in it needs to start at zero, and
// calls whose kernels overlap on the GPU (different streams, or different
// host threads, without ordering between them) race on it.
#include <mutex>

#include "kcommon.cuh"
#include "../../include/qmetal/qmetal_kernels.h"

namespace {

constexpr size_t kScratchBytes = 327 * 1024;
constexpr uint32_t kMaxStateQubits = 34;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_diag_scratch[kScratchBytes];

std::mutex g_lock;
void *g_scratch_addr[kMaxDevices] = {nullptr};

// The array's name is a host-side stand-in in host code; its device address
// is looked up once per device, with that device current, and kept for the
// process (a cudaDeviceReset would drop the array with the context, so the
// entry point is documented as not usable on a device after a reset).
int scratch_for_current_device(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return static_cast<int>(e);
  if (dev < 0 || dev >= kMaxDevices) return -1;
  std::lock_guard<std::mutex> guard(g_lock);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_diag_scratch);
    if (e != cudaSuccess) return static_cast<int>(e);
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return 0;
}

}  // namespace

extern "C" int qmk_apply_diagonal_noalloc(float *state, uint32_t n, uint32_t num_terms,
                                          const uint64_t *masks, const double *angles,
                                          double global_phase, void *stream) {
  if (n > kMaxStateQubits || qmk_workspace_bytes(n) > kScratchBytes) return QMK_ERR_TOO_LARGE;
  void *scratch = nullptr;
  const int rc = scratch_for_current_device(&scratch);
  if (rc != 0) return rc;
  return qmk_apply_diagonal(state, n, num_terms, masks, angles, global_phase, scratch,
                            kScratchBytes, stream);
}
