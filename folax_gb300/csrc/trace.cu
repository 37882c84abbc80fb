// Opt-in kernel tracing (CUDA events on the launching stream).  The reference
// has only wall-clock decorators around its Python methods
// (fol/tools/decoration_functions.py:7-32), which see dispatch time, not
// device time; these events see the kernels themselves.
#include <mutex>
#include <vector>

#include "folgb_internal.cuh"

namespace folgb {
namespace {
struct Pending {
  int kid;
  cudaEvent_t a, b;
};
std::mutex mu;
bool enabled = false;
std::vector<Pending> pending;
std::vector<cudaEvent_t> pool;
int64_t launches[KID_COUNT];
double total_ms[KID_COUNT];
cudaEvent_t open_event[KID_COUNT];

cudaEvent_t get_event() {
  if (!pool.empty()) {
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}
}  // namespace

bool trace_active() {
  std::lock_guard<std::mutex> g(mu);
  return enabled;
}

void trace_begin(int kid, cudaStream_t s) {
  if (!enabled || kid < 0 || kid >= KID_COUNT) return;
  std::lock_guard<std::mutex> g(mu);
  cudaEvent_t e = get_event();
  cudaEventRecord(e, s);
  open_event[kid] = e;
}

void trace_end(int kid, cudaStream_t s) {
  if (!enabled || kid < 0 || kid >= KID_COUNT) return;
  std::lock_guard<std::mutex> g(mu);
  cudaEvent_t e = get_event();
  cudaEventRecord(e, s);
  pending.push_back({kid, open_event[kid], e});
}
}  // namespace folgb

using namespace folgb;

extern "C" int folgb_trace_enable(int32_t on) {
  std::lock_guard<std::mutex> g(mu);
  enabled = on != 0;
  return FOLGB_OK;
}

extern "C" int folgb_trace_reset(void) {
  std::lock_guard<std::mutex> g(mu);
  for (auto& p : pending) {
    pool.push_back(p.a);
    pool.push_back(p.b);
  }
  pending.clear();
  for (int i = 0; i < KID_COUNT; ++i) {
    launches[i] = 0;
    total_ms[i] = 0.0;
  }
  return FOLGB_OK;
}

extern "C" int folgb_trace_read(int32_t kernel_id, int64_t* n_launches, double* ms) {
  if (kernel_id < 0 || kernel_id >= KID_COUNT) return FOLGB_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(mu);
  for (auto& p : pending) {
    FOLGB_CUDA_TRY(cudaEventSynchronize(p.b));
    float t = 0.f;
    FOLGB_CUDA_TRY(cudaEventElapsedTime(&t, p.a, p.b));
    launches[p.kid] += 1;
    total_ms[p.kid] += t;
    pool.push_back(p.a);
    pool.push_back(p.b);
  }
  pending.clear();
  if (n_launches) *n_launches = launches[kernel_id];
  if (ms) *ms = total_ms[kernel_id];
  return FOLGB_OK;
}

// ---------------------------------------------------------------------------
// Self-test of the bounded mbarrier wait that the TMA-staged kernels use:
// one thread initialises a barrier in shared memory, announces 16 bytes of
// transactions that no copy will ever deliver, and waits with
// mbar_wait_bounded.  The wait gives up after its poll limit, the kernel
// records FOLGB_ERR_TIMEOUT in the status word and returns; nothing else is
// pending on the barrier, so the block exits cleanly and the context stays
// usable.
// ---------------------------------------------------------------------------
namespace folgb {
__global__ void k_selftest_bounded_wait(int* status) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  fence_mbar_init();
  mbar_arrive_expect_tx(&bar, 16u);
  if (!mbar_wait_bounded(&bar, 0u)) atomicOr(status, 1 << FOLGB_ERR_TIMEOUT);
}
}  // namespace folgb

extern "C" int folgb_selftest_bounded_wait(int32_t* device_status, void* stream) {
  if (!device_status) return FOLGB_ERR_INVALID_ARGUMENT;
  folgb::k_selftest_bounded_wait<<<1, 32, 0, (cudaStream_t)stream>>>(device_status);
  FOLGB_LAUNCH_CHECK();
  return FOLGB_OK;
}

// ---------------------------------------------------------------------------
// FP32 throughput probe (no counterpart in the reference): a grid of
// independent fused multiply-add chains over every SM, for measuring the FP32
// peak a roofline is reported against.  Each thread runs 8 chains of packed
// fp32 pairs (FFMA2: two IEEE fp32 fused multiply-adds per instruction);
// x <- x * b + c with |b| < 1 stays finite for any iteration count.  The
// result is stored only if it equals a value it never reaches, so the work
// cannot be removed and nothing is written.
// ---------------------------------------------------------------------------
namespace folgb {
constexpr int kPeakThreads = 256, kPeakChains = 8;
__global__ void __launch_bounds__(kPeakThreads) k_fp32_peak(float* sink, int iters, float b0, float c0) {
  float2 acc[kPeakChains];
#pragma unroll
  for (int k = 0; k < kPeakChains; ++k) acc[k] = make_float2(1e-3f * threadIdx.x + k, 0.5f * k);
  const float2 b = make_float2(b0, b0), c = make_float2(c0, c0);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kPeakChains; ++k) acc[k] = __ffma2_rn(acc[k], b, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kPeakChains; ++k) s += acc[k].x + acc[k].y;
  if (s == -1234.5f) sink[0] = s;
}
}  // namespace folgb

extern "C" int folgb_fp32_peak_probe(float* sink, int32_t blocks_per_sm, int32_t iterations,
                                     double* flops_per_launch, void* stream) {
  if (!sink || blocks_per_sm <= 0 || blocks_per_sm > 64 || iterations <= 0) return FOLGB_ERR_INVALID_ARGUMENT;
  const int64_t blocks = (int64_t)blocks_per_sm * num_sms();
  folgb::k_fp32_peak<<<(unsigned)blocks, folgb::kPeakThreads, 0, (cudaStream_t)stream>>>(sink, iterations, 0.999f,
                                                                                          1e-3f);
  FOLGB_LAUNCH_CHECK();
  if (flops_per_launch)
    *flops_per_launch = (double)blocks * folgb::kPeakThreads * iterations * folgb::kPeakChains * 2.0 * 2.0;
  return FOLGB_OK;
}
