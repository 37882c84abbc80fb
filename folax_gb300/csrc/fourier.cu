// Nodal Fourier control on the device: FourierControl.ComputeControlledVariables
// (fol/controls/fourier_control.py:24-59) and its vector-Jacobian product, so a
// training step maps Fourier coefficients to the nodal material field and the
// loss gradient back to the coefficients without leaving the GPU.
//
//   v = coeffs * (scale_max - scale_min) + scale_min            (:51-52)
//   K(x) = v0 / 2 + sum_f v_{1+f} cos(fx pi x) cos(fy pi y) cos(fz pi z)
//   value = (max - min) * sigmoid(beta (K - 0.5)) + min         (:53-59)
// with f running over meshgrid(x_freqs, y_freqs, z_freqs, indexing="ij")
// flattened row-major (:44-45).
//
// Layout: per-node cosine tables cx [nx][N], cy [ny][N], cz [nz][N] (fp32,
// computed on the host in fp64 once), coefficients [B][F+1].  K is evaluated
// sum-factorised, sum_i cx_i (sum_j cy_j (sum_k c_ijk cz_k)).  The backward
// pass reduces over nodes per coefficient into per-block partials and the
// last block sums them in a fixed order (deterministic, no float atomics).
#include <cmath>
#include <vector>

#include "folgb_internal.cuh"

struct folgb_fourier {
  int nx, ny, nz, F;
  int64_t N;
  float vmin, vmax, beta, scale, shift;
  float *d_cx = nullptr, *d_cy = nullptr, *d_cz = nullptr;
};

namespace folgb {

constexpr int kFourierThreads = 256;
constexpr int kFourierChunk = 8;      // coefficients per backward sweep
constexpr int kFourierMaxCoeffs = 8192;

struct FourierArgs {
  int nx, ny, nz, F;
  int64_t N;
  float vmin, vmax, beta, scale, shift;
  const float *cx, *cy, *cz;
};

__device__ __forceinline__ float fourier_K(const FourierArgs& a, const float* __restrict__ c, int64_t n) {
  float K = 0.5f * c[0];
  int f = 1;
  for (int i = 0; i < a.nx; ++i) {
    float si = 0.f;
    for (int j = 0; j < a.ny; ++j) {
      float tij = 0.f;
      for (int k = 0; k < a.nz; ++k, ++f) tij = fmaf(c[f], __ldg(a.cz + (int64_t)k * a.N + n), tij);
      si = fmaf(tij, __ldg(a.cy + (int64_t)j * a.N + n), si);
    }
    K = fmaf(si, __ldg(a.cx + (int64_t)i * a.N + n), K);
  }
  return K;
}

__device__ __forceinline__ float sigmoidf(float t) { return 1.f / (1.f + expf(-t)); }

// coefficients of instance b, scaled, into shared memory
__device__ __forceinline__ void load_coeffs(const FourierArgs& a, const float* __restrict__ coeffs, int b,
                                            float* sc) {
  const float* cb = coeffs + (int64_t)b * (a.F + 1);
  for (int i = threadIdx.x; i <= a.F; i += blockDim.x) sc[i] = fmaf(cb[i], a.scale, a.shift);
  __syncthreads();
}

__global__ void __launch_bounds__(kFourierThreads) k_fourier_forward(const FourierArgs a,
                                                                     const float* __restrict__ coeffs,
                                                                     float* __restrict__ values) {
  extern __shared__ float sc[];
  const int b = blockIdx.y;
  load_coeffs(a, coeffs, b, sc);
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.N) return;
  const float K = fourier_K(a, sc, n);
  values[(int64_t)b * a.N + n] = (a.vmax - a.vmin) * sigmoidf(a.beta * (K - 0.5f)) + a.vmin;
}

// g_n = dvalues_n * dvalue/dK_n = dvalues_n (max - min) beta s (1 - s)
__global__ void __launch_bounds__(kFourierThreads) k_fourier_dK(const FourierArgs a, const float* __restrict__ coeffs,
                                                                const float* __restrict__ dvalues,
                                                                float* __restrict__ g) {
  extern __shared__ float sc[];
  const int b = blockIdx.y;
  load_coeffs(a, coeffs, b, sc);
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.N) return;
  const float s = sigmoidf(a.beta * (fourier_K(a, sc, n) - 0.5f));
  const int64_t i = (int64_t)b * a.N + n;
  g[i] = dvalues[i] * (a.vmax - a.vmin) * a.beta * s * (1.f - s);
}

// dcoeffs[b][q] = scale * sum_n g_n dK_n/dv_q: per-block partials over a
// grid-stride share of the nodes, kFourierChunk coefficients per sweep; the
// last block to finish sums the partials in block order.
__global__ void __launch_bounds__(kFourierThreads) k_fourier_reduce(const FourierArgs a, const float* __restrict__ g,
                                                                    float* __restrict__ dcoeffs, float* partials,
                                                                    unsigned* counters) {
  __shared__ float red[32];
  __shared__ bool last;
  const int b = blockIdx.y;
  const int nblk = gridDim.x;
  const int64_t stride = (int64_t)nblk * blockDim.x;
  const int64_t n0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float* part = partials + ((int64_t)b * nblk + blockIdx.x) * (a.F + 1);
  const float* gb = g + (int64_t)b * a.N;
  for (int q0 = 0; q0 <= a.F; q0 += kFourierChunk) {
    // (i, j, k) of each coefficient of the chunk; q = 0 is the constant term
    const float* px[kFourierChunk];
    const float* py[kFourierChunk];
    const float* pz[kFourierChunk];
#pragma unroll
    for (int t = 0; t < kFourierChunk; ++t) {
      const int f = q0 + t - 1;
      const bool basis = f >= 0 && f < a.F;
      const int i = basis ? f / (a.ny * a.nz) : 0, j = basis ? (f / a.nz) % a.ny : 0, k = basis ? f % a.nz : 0;
      px[t] = a.cx + (int64_t)i * a.N;
      py[t] = a.cy + (int64_t)j * a.N;
      pz[t] = a.cz + (int64_t)k * a.N;
    }
    float acc[kFourierChunk];
#pragma unroll
    for (int t = 0; t < kFourierChunk; ++t) acc[t] = 0.f;
    for (int64_t n = n0; n < a.N; n += stride) {
      const float gn = gb[n];
#pragma unroll
      for (int t = 0; t < kFourierChunk; ++t) {
        const int q = q0 + t;
        const float basis = (q == 0) ? 0.5f : __ldg(px[t] + n) * __ldg(py[t] + n) * __ldg(pz[t] + n);
        if (q <= a.F) acc[t] = fmaf(gn, basis, acc[t]);
      }
    }
#pragma unroll
    for (int t = 0; t < kFourierChunk; ++t) {
      const float v = block_sum(acc[t], red);
      if (threadIdx.x == 0 && q0 + t <= a.F) part[q0 + t] = v;
    }
  }
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(counters + b, 1u) == (unsigned)nblk - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const volatile float* pb = partials + (int64_t)b * nblk * (a.F + 1);
  for (int q = threadIdx.x; q <= a.F; q += blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < nblk; ++k) s += pb[(int64_t)k * (a.F + 1) + q];
    dcoeffs[(int64_t)b * (a.F + 1) + q] = a.scale * s;
  }
  if (threadIdx.x == 0) counters[b] = 0u;  // ready for the next launch
}

static FourierArgs fourier_args(const folgb_fourier* f) {
  FourierArgs a;
  a.nx = f->nx;
  a.ny = f->ny;
  a.nz = f->nz;
  a.F = f->F;
  a.N = f->N;
  a.vmin = f->vmin;
  a.vmax = f->vmax;
  a.beta = f->beta;
  a.scale = f->scale;
  a.shift = f->shift;
  a.cx = f->d_cx;
  a.cy = f->d_cy;
  a.cz = f->d_cz;
  return a;
}

static int fourier_blocks(const folgb_fourier* f) {
  int64_t blocks = (f->N + kFourierThreads - 1) / kFourierThreads;
  int64_t cap = (int64_t)num_sms() * 2;
  return (int)(blocks < cap ? blocks : cap);
}

static size_t layout_fourier(const folgb_fourier* f, int32_t B, void* base, size_t cap, float** g,
                             float** partials, unsigned** counters) {
  Bump bp(base, cap);
  float* gg = bp.take<float>((size_t)B * f->N);
  float* p = bp.take<float>((size_t)B * fourier_blocks(f) * (f->F + 1));
  unsigned* c = bp.take<unsigned>((size_t)B);
  if (g) *g = gg;
  if (partials) *partials = p;
  if (counters) *counters = c;
  return align_up(bp.off);
}

}  // namespace folgb

using namespace folgb;

extern "C" int folgb_fourier_create(folgb_fourier** out, const double* x_freqs, int32_t nx, const double* y_freqs,
                                    int32_t ny, const double* z_freqs, int32_t nz, const double* xyz,
                                    int64_t num_nodes, double min_value, double max_value, double beta,
                                    double scale_min, double scale_max) {
  if (!out || !x_freqs || !y_freqs || !z_freqs || !xyz || nx <= 0 || ny <= 0 || nz <= 0 || num_nodes <= 0)
    return FOLGB_ERR_INVALID_ARGUMENT;
  if ((int64_t)nx * ny * nz + 1 > kFourierMaxCoeffs) return FOLGB_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  folgb_fourier* f = new folgb_fourier();
  f->nx = nx;
  f->ny = ny;
  f->nz = nz;
  f->F = nx * ny * nz;
  f->N = num_nodes;
  f->vmin = (float)min_value;
  f->vmax = (float)max_value;
  f->beta = (float)beta;
  f->scale = (float)(scale_max - scale_min);
  f->shift = (float)scale_min;
  const double pi = 3.14159265358979323846;
  auto table = [&](const double* fr, int m, int axis, float** dptr) -> int {
    std::vector<float> h((size_t)m * num_nodes);
    for (int i = 0; i < m; ++i)
      for (int64_t n = 0; n < num_nodes; ++n) h[(size_t)i * num_nodes + n] = (float)std::cos(fr[i] * pi * xyz[3 * n + axis]);
    FOLGB_CUDA_TRY(cudaMalloc(dptr, h.size() * sizeof(float)));
    FOLGB_CUDA_TRY(cudaMemcpy(*dptr, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    return FOLGB_OK;
  };
  int rc = table(x_freqs, nx, 0, &f->d_cx);
  if (!rc) rc = table(y_freqs, ny, 1, &f->d_cy);
  if (!rc) rc = table(z_freqs, nz, 2, &f->d_cz);
  if (rc) {
    folgb_fourier_destroy(f);
    return rc;
  }
  *out = f;
  return FOLGB_OK;
}

extern "C" int folgb_fourier_destroy(folgb_fourier* f) {
  if (!f) return FOLGB_OK;
  cudaFree(f->d_cx);
  cudaFree(f->d_cy);
  cudaFree(f->d_cz);
  delete f;
  return FOLGB_OK;
}

extern "C" size_t folgb_fourier_workspace_bytes(const folgb_fourier* f, int32_t batch) {
  if (!f || batch <= 0) return 0;
  return layout_fourier(f, batch, nullptr, 0, nullptr, nullptr, nullptr);
}

extern "C" int folgb_fourier_forward(const folgb_fourier* f, int32_t batch, const float* coeffs, float* values,
                                     void* stream) {
  if (!f || batch <= 0 || !coeffs || !values) return FOLGB_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  dim3 grid((unsigned)((f->N + kFourierThreads - 1) / kFourierThreads), (unsigned)batch);
  const size_t smem = sizeof(float) * (f->F + 1);
  if (smem > 48 * 1024)
    FOLGB_CUDA_TRY(cudaFuncSetAttribute(k_fourier_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_fourier_forward<<<grid, kFourierThreads, smem, s>>>(fourier_args(f), coeffs, values);
  FOLGB_LAUNCH_CHECK();
  return FOLGB_OK;
}

extern "C" int folgb_fourier_backward(const folgb_fourier* f, int32_t batch, const float* coeffs,
                                      const float* dvalues, float* dcoeffs, void* workspace, size_t workspace_bytes,
                                      void* stream) {
  if (!f || batch <= 0 || !coeffs || !dvalues || !dcoeffs) return FOLGB_ERR_INVALID_ARGUMENT;
  float *g, *partials;
  unsigned* counters;
  const size_t need = layout_fourier(f, batch, workspace, workspace_bytes, &g, &partials, &counters);
  if (!workspace || workspace_bytes < need) return FOLGB_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  FOLGB_CUDA_TRY(cudaMemsetAsync(counters, 0, sizeof(unsigned) * batch, s));
  const size_t smem = sizeof(float) * (f->F + 1);
  if (smem > 48 * 1024)
    FOLGB_CUDA_TRY(cudaFuncSetAttribute(k_fourier_dK, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const FourierArgs a = fourier_args(f);
  k_fourier_dK<<<dim3((unsigned)((f->N + kFourierThreads - 1) / kFourierThreads), (unsigned)batch),
                 kFourierThreads, smem, s>>>(a, coeffs, dvalues, g);
  FOLGB_LAUNCH_CHECK();
  k_fourier_reduce<<<dim3((unsigned)fourier_blocks(f), (unsigned)batch), kFourierThreads, 0, s>>>(a, g, dcoeffs,
                                                                                                  partials, counters);
  FOLGB_LAUNCH_CHECK();
  return FOLGB_OK;
}
