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

constexpr int kFourierTile = 4;        // frequencies per axis of a tile
constexpr int kFourierTiledMax = 64;   // tiles the forward kernels keep padded in shared memory

// Tiled evaluation, for bases of at most kFourierTiledMax tiles: shared memory
// holds the scaled coefficients padded to tiles of 4 x 4 x 4 (zeros for
// frequencies past an edge), sp[64 t + (i 4 + j) 4 + k], and sp[64 T] the
// constant term.  A node then loads its 12 table values of a tile once and
// contracts k with one 16-byte shared load per (i, j).
__device__ __forceinline__ int fourier_tiles_y(const FourierArgs& a) { return (a.ny + kFourierTile - 1) / kFourierTile; }
__device__ __forceinline__ int fourier_tiles_z(const FourierArgs& a) { return (a.nz + kFourierTile - 1) / kFourierTile; }

__device__ __forceinline__ float fourier_K_tiled(const FourierArgs& a, const float* __restrict__ sp, int tiles,
                                                 int64_t n) {
  constexpr int M = kFourierTile;
  const int ty = fourier_tiles_y(a), tz = fourier_tiles_z(a);
  float K = 0.5f * sp[M * M * M * tiles];
  for (int t = 0; t < tiles; ++t) {
    const int i0 = M * (t / (ty * tz)), j0 = M * ((t / tz) % ty), k0 = M * (t % tz);
    float cx[M], cy[M], cz[M];
#pragma unroll
    for (int i = 0; i < M; ++i) {
      cx[i] = i0 + i < a.nx ? __ldg(a.cx + (int64_t)(i0 + i) * a.N + n) : 0.f;
      cy[i] = j0 + i < a.ny ? __ldg(a.cy + (int64_t)(j0 + i) * a.N + n) : 0.f;
      cz[i] = k0 + i < a.nz ? __ldg(a.cz + (int64_t)(k0 + i) * a.N + n) : 0.f;
    }
    const float4* ct = reinterpret_cast<const float4*>(sp + M * M * M * t);
#pragma unroll
    for (int i = 0; i < M; ++i) {
      float si = 0.f;
#pragma unroll
      for (int j = 0; j < M; ++j) {
        const float4 c = ct[i * M + j];
        const float tij = fmaf(c.w, cz[3], fmaf(c.z, cz[2], fmaf(c.y, cz[1], c.x * cz[0])));
        si = fmaf(tij, cy[j], si);
      }
      K = fmaf(si, cx[i], K);
    }
  }
  return K;
}

// coefficients of instance b, scaled, into shared memory: padded tiles
// (tiles > 0) or the plain order (tiles == 0)
__device__ __forceinline__ void load_coeffs(const FourierArgs& a, const float* __restrict__ coeffs, int b,
                                            int tiles, float* sc) {
  const float* cb = coeffs + (int64_t)b * (a.F + 1);
  if (tiles == 0) {
    for (int i = threadIdx.x; i <= a.F; i += blockDim.x) sc[i] = fmaf(cb[i], a.scale, a.shift);
  } else {
    constexpr int M = kFourierTile;
    const int ty = fourier_tiles_y(a), tz = fourier_tiles_z(a);
    for (int p = threadIdx.x; p <= M * M * M * tiles; p += blockDim.x) {
      int q = 0;  // p == 64 T: the constant term
      if (p < M * M * M * tiles) {
        const int t = p / (M * M * M), slot = p % (M * M * M);
        const int i = M * (t / (ty * tz)) + slot / (M * M), j = M * ((t / tz) % ty) + (slot / M) % M,
                  k = M * (t % tz) + slot % M;
        q = (i < a.nx && j < a.ny && k < a.nz) ? 1 + (i * a.ny + j) * a.nz + k : -1;
      }
      sc[p] = q < 0 ? 0.f : fmaf(cb[q], a.scale, a.shift);
    }
  }
  __syncthreads();
}

__device__ __forceinline__ float fourier_K_any(const FourierArgs& a, const float* sc, int tiles, int64_t n) {
  return tiles > 0 ? fourier_K_tiled(a, sc, tiles, n) : fourier_K(a, sc, n);
}

__global__ void __launch_bounds__(kFourierThreads) k_fourier_forward(const FourierArgs a,
                                                                     const float* __restrict__ coeffs,
                                                                     float* __restrict__ values, int tiles) {
  extern __shared__ float4 sc4[];
  float* sc = reinterpret_cast<float*>(sc4);
  const int b = blockIdx.y;
  load_coeffs(a, coeffs, b, tiles, sc);
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.N) return;
  const float K = fourier_K_any(a, sc, tiles, n);
  values[(int64_t)b * a.N + n] = (a.vmax - a.vmin) * sigmoidf(a.beta * (K - 0.5f)) + a.vmin;
}

// g_n = dvalues_n * dvalue/dK_n = dvalues_n (max - min) beta s (1 - s)
__global__ void __launch_bounds__(kFourierThreads) k_fourier_dK(const FourierArgs a, const float* __restrict__ coeffs,
                                                                const float* __restrict__ dvalues,
                                                                float* __restrict__ g, int tiles) {
  extern __shared__ float4 sc4[];
  float* sc = reinterpret_cast<float*>(sc4);
  const int b = blockIdx.y;
  load_coeffs(a, coeffs, b, tiles, sc);
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.N) return;
  const float s = sigmoidf(a.beta * (fourier_K_any(a, sc, tiles, n) - 0.5f));
  const int64_t i = (int64_t)b * a.N + n;
  g[i] = dvalues[i] * (a.vmax - a.vmin) * a.beta * s * (1.f - s);
}

// dcoeffs[b][q] = scale * sum_n g_n dK_n/dv_q, with dK/dv_0 = 1/2 and
// dK/dv_(1+f) = cx_i cy_j cz_k for f = (i ny + j) nz + k.  The frequency grid
// is cut into tiles of kFourierTile^3 (blockIdx.z; unused frequencies of an
// edge tile read as 0) and each block makes one pass over its grid-stride
// share of the nodes, keeping all 64 sums of its tile in registers:
// h_jk = g cy_j cz_k, acc_ijk += cx_i h_jk (12 table loads and 80 FMAs a
// node).  A warp reduces its 64 sums by halving: at each shuffle step a lane
// keeps one half of its values (the upper half when its lane bit for that
// step is set) and adds the partner's copy of that half, so 62 shuffles leave
// lane L holding sums 2L and 2L + 1.  The block adds its warps' sums in warp
// order into its row of partials, and the last block of instance b (over all
// tiles) sums the rows in block order: a fixed order, no float atomics.

template <int C, int O>
__device__ __forceinline__ void fourier_halving(float (&v)[64], int lane) {
  if constexpr (C > 2 || (C == 2 && O >= 1)) {
    const bool up = (lane & O) != 0;
#pragma unroll
    for (int k = 0; k < C / 2; ++k) {
      const float send = up ? v[k] : v[k + C / 2];
      const float keep = up ? v[k + C / 2] : v[k];
      v[k] = keep + __shfl_xor_sync(0xffffffffu, send, O);
    }
    if constexpr (O > 1) fourier_halving<C / 2, O / 2>(v, lane);
  }
}

__global__ void __launch_bounds__(kFourierThreads) k_fourier_reduce(const FourierArgs a, const float* __restrict__ g,
                                                                    float* __restrict__ dcoeffs, float* partials,
                                                                    unsigned* counters) {
  constexpr int M = kFourierTile, NW = kFourierThreads / 32;
  __shared__ float wsum[NW][M * M * M + 1];
  __shared__ bool last;
  const int b = blockIdx.y, nblk = gridDim.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int tiles_y = fourier_tiles_y(a), tiles_z = fourier_tiles_z(a);
  const int i0 = M * (int)(blockIdx.z / (tiles_y * tiles_z)), j0 = M * (int)((blockIdx.z / tiles_z) % tiles_y),
            k0 = M * (int)(blockIdx.z % tiles_z);
  const int64_t stride = (int64_t)nblk * blockDim.x;
  const float* gb = g + (int64_t)b * a.N;
  float acc[M * M * M];
#pragma unroll
  for (int t = 0; t < M * M * M; ++t) acc[t] = 0.f;
  float acc0 = 0.f;
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < a.N; n += stride) {
    const float gn = gb[n];
    float cx[M], cy[M], cz[M];
#pragma unroll
    for (int i = 0; i < M; ++i) {
      cx[i] = i0 + i < a.nx ? __ldg(a.cx + (int64_t)(i0 + i) * a.N + n) : 0.f;
      cy[i] = j0 + i < a.ny ? __ldg(a.cy + (int64_t)(j0 + i) * a.N + n) : 0.f;
      cz[i] = k0 + i < a.nz ? __ldg(a.cz + (int64_t)(k0 + i) * a.N + n) : 0.f;
    }
    acc0 += gn;
#pragma unroll
    for (int j = 0; j < M; ++j)
#pragma unroll
      for (int k = 0; k < M; ++k) {
        const float h = gn * cy[j] * cz[k];
#pragma unroll
        for (int i = 0; i < M; ++i) acc[(i * M + j) * M + k] = fmaf(cx[i], h, acc[(i * M + j) * M + k]);
      }
  }
  fourier_halving<M * M * M, 16>(acc, lane);
  wsum[warp][2 * lane] = acc[0];
  wsum[warp][2 * lane + 1] = acc[1];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc0 += __shfl_xor_sync(0xffffffffu, acc0, o);
  if (lane == 0) wsum[warp][M * M * M] = acc0;
  __syncthreads();
  // this tile's coefficients of the block's row (the constant term from tile 0)
  float* part = partials + ((int64_t)b * nblk + blockIdx.x) * (a.F + 1);
  for (int slot = threadIdx.x; slot <= M * M * M; slot += blockDim.x) {
    int q;
    if (slot == M * M * M) {
      q = blockIdx.z == 0 ? 0 : -1;
    } else {
      const int i = i0 + slot / (M * M), j = j0 + (slot / M) % M, k = k0 + slot % M;
      q = (i < a.nx && j < a.ny && k < a.nz) ? 1 + (i * a.ny + j) * a.nz + k : -1;
    }
    if (q < 0) continue;
    float v = 0.f;
#pragma unroll
    for (int w = 0; w < NW; ++w) v += wsum[w][slot];
    part[q] = q == 0 ? 0.5f * v : v;
  }
  __threadfence();  // every writer's partials are visible before the block is counted
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counters + b, 1u) == (unsigned)(nblk * gridDim.z) - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  const volatile float* pb = partials + (int64_t)b * nblk * (a.F + 1);
  for (int q = threadIdx.x; q <= a.F; q += blockDim.x) {
    float sum = 0.f;
    for (int k = 0; k < nblk; ++k) sum += pb[(int64_t)k * (a.F + 1) + q];
    dcoeffs[(int64_t)b * (a.F + 1) + q] = a.scale * sum;
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

static int fourier_tiles(const folgb_fourier* f) {
  auto t = [](int m) { return (m + kFourierTile - 1) / kFourierTile; };
  return t(f->nx) * t(f->ny) * t(f->nz);
}

// tiles of the padded shared-memory layout, or 0 for the plain order
static int fourier_forward_tiles(const folgb_fourier* f) {
  const int t = fourier_tiles(f);
  return t <= kFourierTiledMax ? t : 0;
}

static size_t fourier_forward_smem(const folgb_fourier* f) {
  const int t = fourier_forward_tiles(f);
  return sizeof(float) * (t > 0 ? (size_t)kFourierTile * kFourierTile * kFourierTile * t + 4 : (size_t)f->F + 1);
}

// blocks per (instance, tile): two per SM for one tile, fewer per tile when
// there are several (at least 32, for load balance), never more than the nodes need
static int fourier_blocks(const folgb_fourier* f) {
  int64_t blocks = (f->N + kFourierThreads - 1) / kFourierThreads;
  int64_t cap = (int64_t)num_sms() * 2 / fourier_tiles(f);
  if (cap < 32) cap = 32;
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
  const int tiles = fourier_forward_tiles(f);
  const size_t smem = fourier_forward_smem(f);
  if (smem > 48 * 1024)
    FOLGB_CUDA_TRY(cudaFuncSetAttribute(k_fourier_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_fourier_forward<<<grid, kFourierThreads, smem, s>>>(fourier_args(f), coeffs, values, tiles);
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
  const int tiles = fourier_forward_tiles(f);
  const size_t smem = fourier_forward_smem(f);
  if (smem > 48 * 1024)
    FOLGB_CUDA_TRY(cudaFuncSetAttribute(k_fourier_dK, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const FourierArgs a = fourier_args(f);
  k_fourier_dK<<<dim3((unsigned)((f->N + kFourierThreads - 1) / kFourierThreads), (unsigned)batch),
                 kFourierThreads, smem, s>>>(a, coeffs, dvalues, g, tiles);
  FOLGB_LAUNCH_CHECK();
  k_fourier_reduce<<<dim3((unsigned)fourier_blocks(f), (unsigned)batch, (unsigned)fourier_tiles(f)),
                     kFourierThreads, 0, s>>>(a, g, dcoeffs, partials, counters);
  FOLGB_LAUNCH_CHECK();
  return FOLGB_OK;
}
