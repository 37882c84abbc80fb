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
//   * the array's device address is looked up (cudaGetSymbolAddress, with
//     the device current) when the first plan is created on a device
//     (folgb_plan_create).  With lazy module loading that lookup is what
//     loads this file's module and commits the 48 MiB, so it happens at plan
//     creation, where the caller is allocating anyway, and never inside a
//     no-alloc call on a device that has a plan.  The address is cached per
//     device together with the id of the CUDA context it belongs to; a call
//     made under a different context (after cudaDeviceReset, or a primary
//     context that was released and made again) looks it up again;
//   * create the plans before any CUDA stream capture.
//
// Everything else (status codes, outputs, semantics) is folgb_loss_adjoint's.
#include <cuda.h>  // CUcontext / CUresult types; the two driver calls come from the runtime's entry-point table

#include <mutex>

#include "folgb_internal.cuh"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(48) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// Unique id of the calling thread's current CUDA context (cuCtxGetId, which
// never repeats within a process, unlike a context handle).  Called with
// g_setup_mutex held.
int current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void *f1 = nullptr, *f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return FOLGB_ERR_CUDA;
    get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, id) != CUDA_SUCCESS) return FOLGB_ERR_CUDA;
  return FOLGB_OK;
}

// Device address of g_noalloc_scratch on the current device, looked up when
// the device's cached address is missing or belongs to another context.
int scratch_address(void** out) {
  int dev = 0;
  FOLGB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return FOLGB_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  unsigned long long ctx = 0;
  const bool have_ctx = g_scratch_ptr[dev] && current_context_id(&ctx) == FOLGB_OK;
  if (!have_ctx || ctx != g_scratch_ctx[dev]) {
    void* ptr = nullptr;
    cudaError_t err = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (err != cudaSuccess || ptr == nullptr) {
      (void)cudaGetLastError();  // a failed module load (out of memory) is not sticky
      fprintf(stderr, "folgb: cudaGetSymbolAddress(no-alloc scratch) failed on device %d: %s\n", dev,
              cudaGetErrorString(err));
      g_scratch_ptr[dev] = nullptr;
      return FOLGB_ERR_CUDA;
    }
    int rc = current_context_id(&ctx);  // the lookup made the context current if it was not
    if (rc) return rc;
    g_scratch_ptr[dev] = ptr;
    g_scratch_ctx[dev] = ctx;
  }
  *out = g_scratch_ptr[dev];
  return FOLGB_OK;
}

}  // namespace

namespace folgb {
// Called by folgb_plan_create with the plan's device current: commits the
// scratch array there (see the file comment).  A failure is not an error of
// the plan: the no-alloc call retries the lookup and reports it.
void noalloc_prepare_current_device() {
  void* ptr = nullptr;
  (void)scratch_address(&ptr);
}
}  // namespace folgb

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
