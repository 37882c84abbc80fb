// Fused loss + adjoint for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc (or any allocator) at
// the point where they evaluate the loss: a framework custom call whose
// buffers are all planned by the framework and which has no scratch-buffer
// slot to ask for; code that runs under a memory budget reserved up front;
// code called from inside an allocator hook, where allocating again would
// re-enter the allocator.  folgb_loss_adjoint needs a caller-provided
// workspace; folgb_loss_adjoint_noalloc instead uses a fixed scratch array
// that is part of this library's device image:
//
//   * kNoAllocScratchBytes (48 MiB) of device memory, held by every GPU that
//     loads the library until the process exits;
//   * enough for the hex8 elasticity loss on a 64^3 mesh (batch 1); larger
//     problems are rejected with FOLGB_ERR_TOO_LARGE before any work;
//   * one array per device, shared by every call: calls whose work overlaps
//     on the GPU (two streams, two threads) race on it.  Order them on one
//     stream.  Each call clears the parts that must start at zero and
//     overwrites the rest;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current) and caches it; make
//     that first call before any CUDA stream capture.
//
// Everything else (status codes, outputs, semantics) is folgb_loss_adjoint's.
#include <mutex>

#include "folgb_internal.cuh"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(48) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once).
int scratch_address(void** out) {
  int dev = 0;
  FOLGB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return FOLGB_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* ptr = nullptr;
    cudaError_t err = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (err != cudaSuccess || ptr == nullptr) {
      fprintf(stderr, "folgb: cudaGetSymbolAddress(no-alloc scratch) failed on device %d: %s\n", dev,
              cudaGetErrorString(err));
      return FOLGB_ERR_CUDA;
    }
    g_scratch_ptr[dev] = ptr;
  }
  *out = g_scratch_ptr[dev];
  return FOLGB_OK;
}

}  // namespace

extern "C" int folgb_loss_adjoint_noalloc(const folgb_plan* plan, int32_t batch, const float* control,
                                          int64_t control_stride, const float* dofs, int64_t dofs_stride,
                                          int32_t apply_dirichlet, float* losses, float* dloss_ddofs,
                                          float* dloss_dcontrol, int32_t* device_status, void* stream) {
  if (!plan || batch <= 0) return FOLGB_ERR_INVALID_ARGUMENT;
  const size_t need = folgb_workspace_bytes(plan, FOLGB_OP_LOSS_ADJOINT, batch);
  if (need == 0 || need > kNoAllocScratchBytes) {
    fprintf(stderr, "folgb: loss needs %zu bytes of scratch, the no-alloc entry point has %zu\n", need,
            kNoAllocScratchBytes);
    return FOLGB_ERR_TOO_LARGE;
  }
  void* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc) return rc;
  return folgb_loss_adjoint(plan, batch, control, control_stride, dofs, dofs_stride, apply_dirichlet, losses,
                            dloss_ddofs, dloss_dcontrol, device_status, scratch, kNoAllocScratchBytes, stream);
}
