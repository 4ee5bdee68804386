// fsm_integrate_static: the fused integrate for callers that cannot allocate
// device memory (no cudaMalloc, no allocating library call, no caching
// allocator of their own), for example code running inside a host callback,
// a plugin sandbox that forbids allocation after start-up, or a real-time
// loop that must not block on the allocator. The scratch the column/row
// passes need (the scheme's running sums, the stage fields between the two
// passes, the products) lives in one file-scope device array of
// FSM_STATIC_SCRATCH_BYTES that every GPU loading this library holds until
// the process exits.
#include <mutex>

#include "fsm_internal.cuh"

namespace {

static __device__ __align__(256) unsigned char g_static_scratch[FSM_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device. The host-side
// name g_static_scratch is only a stand-in for the symbol, never a usable
// pointer: the address is looked up once per device, with that device
// current, and cached for the life of the process (a device reset after the
// first call would leave the cached address stale; resets are not supported).
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fsm::cuda_check(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fsm::set_error(FSM_ERR_UNSUPPORTED, "device index out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return fsm::cuda_check(e, "cudaGetSymbolAddress(static scratch)");
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return FSM_OK;
}

}  // namespace

extern "C" int fsm_integrate_static(const FsmPlan* plan, int32_t batch, void* state, int32_t steps, void* stream) {
  if (!plan || !state || batch < 1 || steps < 0) return fsm::set_error(FSM_ERR_INVALID, "integrate_static arguments");
  const size_t need = fsm::integrate_workspace_bytes(plan, batch, steps);
  if (need > (size_t)FSM_STATIC_SCRATCH_BYTES)
    return fsm::set_error(FSM_ERR_INVALID,
                          "fsm_integrate_static: this batch needs " + std::to_string(need) +
                              " bytes of scratch, above the static limit of " +
                              std::to_string((size_t)FSM_STATIC_SCRATCH_BYTES) +
                              " bytes; use fsm_integrate with a caller workspace or a smaller batch");
  void* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc) return rc;
  // Nothing in the scratch has to start at zero: every array is written before it is read.
  return fsm::integrate_with_workspace(plan, batch, state, steps, scratch, (size_t)FSM_STATIC_SCRATCH_BYTES,
                                       (cudaStream_t)stream);
}
