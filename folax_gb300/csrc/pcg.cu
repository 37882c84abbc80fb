// Jacobi-preconditioned CG on the plan's fixed CSR pattern, SpMV, and the
// Adam update.  Replaces FiniteElementSolver.LinearSolve
// (fol/solvers/fe_solver.py:60-78; BiCGSTAB / direct there).
//
// SpMV reads the canonical CSR values but indexes columns through the node
// adjacency (one column index per ndof x ndof block), so the index stream is
// 1/ndof^2 of a scalar CSR's.  One group of G lanes handles one node's ndof
// rows; lane j of the group owns neighbour j.
//
// Each PCG iteration is two kernels:
//   k_pcg_spmv:   p_new = z + beta p_old (formed on the fly at every column),
//                 q = A p_new, partial p_new.q (fp64)  -> alpha (last block)
//   k_pcg_update: x += alpha p_new, r -= alpha q, z = D^-1 r,
//                 partial r.z, r.r (fp64) -> beta, convergence (last block)
// Every kernel returns at once when the device "done" flag is set, so the
// host can enqueue a chunk of iterations and read the flag once per chunk.
#include <cmath>
#include <type_traits>

#include "folgb_internal.cuh"

using namespace folgb;

namespace folgb {

struct PCGScalars {
  double rho;      // r.z of the current iterate
  double pq;       // p.q
  double bnorm2;   // ||b||^2
  double rnorm2;   // ||r||^2
  double tol2;     // rtol^2 ||b||^2
  float alpha, beta;
  int iters;
  int done;        // 1 converged, 2 maxiter, 3 breakdown/non-finite
  int maxiter;
  int pad;
};

struct PCGWork {
  float *r, *z, *p0, *p1, *q;
  double* part;        // [2][maxblocks]
  unsigned* counters;  // [4]
  PCGScalars* sc;
};

constexpr int kVecBlocks = 1024;  // grid cap for vector kernels (multiple of the SM count not needed)

static size_t layout_pcg(const folgb_plan* p, void* base, size_t cap, PCGWork* w) {
  Bump bp(base, cap);
  const size_t n = (size_t)p->ndof * p->N;
  PCGWork t;
  t.r = bp.take<float>(n);
  t.z = bp.take<float>(n);
  t.p0 = bp.take<float>(n);
  t.p1 = bp.take<float>(n);
  t.q = bp.take<float>(n);
  t.part = bp.take<double>(2 * 65536);
  t.counters = bp.take<unsigned>(4);
  t.sc = bp.take<PCGScalars>(1);
  if (w) *w = t;
  return align_up(bp.off);
}

size_t pcg_workspace_bytes(const folgb_plan* p) { return layout_pcg(p, nullptr, 0, nullptr); }

// last-block-done helper for fp64 partials; returns true in the last block
__device__ __forceinline__ bool last_block(unsigned* counter) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned prev = atomicAdd(counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  return last;
}

__device__ __forceinline__ double sum_partials(const double* part, int n, double* sh) {
  double s = 0.0;
  const volatile double* pv = part;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += pv[i];
  return block_sum_d(s, sh);
}

__global__ void k_pcg_init(int64_t n, const float* __restrict__ b, const float* __restrict__ dinv, float* __restrict__ x,
                           float* __restrict__ r, float* __restrict__ z, float* __restrict__ p0, double* part,
                           unsigned* counters, PCGScalars* sc, double rtol, int maxiter) {
  __shared__ double sh[32];
  double rz = 0.0, bb = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float bi = b[i];
    float zi = dinv[i] * bi;
    x[i] = 0.f;
    r[i] = bi;
    z[i] = zi;
    p0[i] = 0.f;
    rz += (double)bi * (double)zi;
    bb += (double)bi * (double)bi;
  }
  double s1 = block_sum_d(rz, sh);
  double s2 = block_sum_d(bb, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = s1;
    part[gridDim.x + blockIdx.x] = s2;
  }
  if (!last_block(&counters[0])) return;
  double RZ = sum_partials(part, gridDim.x, sh);
  double BB = sum_partials(part + gridDim.x, gridDim.x, sh);
  if (threadIdx.x == 0) {
    sc->rho = RZ;
    sc->bnorm2 = BB;
    sc->rnorm2 = BB;
    sc->tol2 = rtol * rtol * BB;
    sc->beta = 0.f;
    sc->alpha = 0.f;
    sc->iters = 0;
    sc->maxiter = maxiter;
    sc->done = (BB == 0.0) ? 1 : 0;
    counters[0] = 0u;
  }
}

template <int NDOF, int G>
__global__ void __launch_bounds__(256) k_pcg_spmv(int64_t N, const int* __restrict__ adj_ptr,
                                                  const int* __restrict__ adj, const int* __restrict__ rowptr,
                                                  const float* __restrict__ vals, const float* __restrict__ z,
                                                  const float* __restrict__ pold, float* __restrict__ pnew,
                                                  float* __restrict__ q, double* part, unsigned* counters,
                                                  PCGScalars* sc) {
  __shared__ double sh[32];
  if (sc->done) return;
  const float beta = sc->beta;
  const int lane = threadIdx.x % G;
  const int64_t group = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;
  double dot = 0.0;
  // warp-uniform loop: every lane runs the same number of rounds so the
  // group shuffles below always see the whole warp
  for (int64_t n = group; __any_sync(0xffffffffu, n < N); n += ngroups) {
    const bool active = n < N;
    const int a0 = active ? __ldg(adj_ptr + n) : 0;
    const int deg = active ? __ldg(adj_ptr + n + 1) - a0 : 0;
    float acc[NDOF];
#pragma unroll
    for (int i = 0; i < NDOF; ++i) acc[i] = 0.f;
    int rb[NDOF];
#pragma unroll
    for (int i = 0; i < NDOF; ++i) rb[i] = active ? __ldg(rowptr + (int64_t)NDOF * n + i) : 0;
    for (int j = lane; j < deg; j += G) {
      const int m = __ldg(adj + a0 + j);
      float pv[NDOF];
#pragma unroll
      for (int l = 0; l < NDOF; ++l) pv[l] = fmaf(beta, __ldg(pold + (int64_t)NDOF * m + l), __ldg(z + (int64_t)NDOF * m + l));
#pragma unroll
      for (int i = 0; i < NDOF; ++i)
#pragma unroll
        for (int l = 0; l < NDOF; ++l) acc[i] = fmaf(__ldg(vals + rb[i] + NDOF * j + l), pv[l], acc[i]);
    }
#pragma unroll
    for (int i = 0; i < NDOF; ++i)
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o, G);
    if (active && lane == 0) {
#pragma unroll
      for (int i = 0; i < NDOF; ++i) {
        const int64_t d = (int64_t)NDOF * n + i;
        const float pn = fmaf(beta, pold[d], z[d]);
        pnew[d] = pn;
        q[d] = acc[i];
        dot += (double)pn * (double)acc[i];
      }
    }
  }
  double s = block_sum_d(dot, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  if (!last_block(&counters[1])) return;
  double PQ = sum_partials(part, gridDim.x, sh);
  if (threadIdx.x == 0) {
    sc->pq = PQ;
    if (!(PQ > 0.0) || !isfinite(PQ)) {
      sc->done = 3;
      sc->alpha = 0.f;
    } else {
      sc->alpha = (float)(sc->rho / PQ);
    }
    counters[1] = 0u;
  }
}

__global__ void __launch_bounds__(256) k_pcg_update(int64_t n, const float* __restrict__ dinv, float* __restrict__ x,
                                                    float* __restrict__ r, float* __restrict__ z,
                                                    const float* __restrict__ p, const float* __restrict__ q,
                                                    double* part, unsigned* counters, PCGScalars* sc) {
  __shared__ double sh[32];
  if (sc->done) return;
  const float alpha = sc->alpha;
  double rz = 0.0, rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = fmaf(alpha, p[i], x[i]);
    const float ri = fmaf(-alpha, q[i], r[i]);
    r[i] = ri;
    const float zi = dinv[i] * ri;
    z[i] = zi;
    rz += (double)ri * (double)zi;
    rr += (double)ri * (double)ri;
  }
  double s1 = block_sum_d(rz, sh);
  double s2 = block_sum_d(rr, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = s1;
    part[gridDim.x + blockIdx.x] = s2;
  }
  if (!last_block(&counters[2])) return;
  double RZ = sum_partials(part, gridDim.x, sh);
  double RR = sum_partials(part + gridDim.x, gridDim.x, sh);
  if (threadIdx.x == 0) {
    sc->beta = (float)(RZ / sc->rho);
    sc->rho = RZ;
    sc->rnorm2 = RR;
    sc->iters += 1;
    if (!isfinite(RR)) sc->done = 3;
    else if (RR <= sc->tol2) sc->done = 1;
    else if (sc->iters >= sc->maxiter) sc->done = 2;
    counters[2] = 0u;
  }
}

template <int NDOF, int G>
__global__ void __launch_bounds__(256) k_spmv(int64_t N, const int* __restrict__ adj_ptr, const int* __restrict__ adj,
                                              const int* __restrict__ rowptr, const float* __restrict__ vals,
                                              const float* __restrict__ x, float* __restrict__ y) {
  const int lane = threadIdx.x % G;
  const int64_t group = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;
  for (int64_t n = group; __any_sync(0xffffffffu, n < N); n += ngroups) {
    const bool active = n < N;
    const int a0 = active ? __ldg(adj_ptr + n) : 0;
    const int deg = active ? __ldg(adj_ptr + n + 1) - a0 : 0;
    float acc[NDOF];
#pragma unroll
    for (int i = 0; i < NDOF; ++i) acc[i] = 0.f;
    int rb[NDOF];
#pragma unroll
    for (int i = 0; i < NDOF; ++i) rb[i] = active ? __ldg(rowptr + (int64_t)NDOF * n + i) : 0;
    for (int j = lane; j < deg; j += G) {
      const int m = __ldg(adj + a0 + j);
#pragma unroll
      for (int i = 0; i < NDOF; ++i)
#pragma unroll
        for (int l = 0; l < NDOF; ++l)
          acc[i] = fmaf(__ldg(vals + rb[i] + NDOF * j + l), __ldg(x + (int64_t)NDOF * m + l), acc[i]);
    }
#pragma unroll
    for (int i = 0; i < NDOF; ++i)
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o, G);
    if (active && lane == 0) {
#pragma unroll
      for (int i = 0; i < NDOF; ++i) y[(int64_t)NDOF * n + i] = acc[i];
    }
  }
}

template <int NDOF>
static int group_width(int maxdeg) {
  int g = 1;
  while (g < maxdeg && g < 32) g <<= 1;
  return g < 4 ? 4 : g;
}

template <int NDOF, class F>
static int with_group(int maxdeg, F&& f) {
  switch (group_width<NDOF>(maxdeg)) {
    case 4: return f(std::integral_constant<int, 4>{});
    case 8: return f(std::integral_constant<int, 8>{});
    case 16: return f(std::integral_constant<int, 16>{});
    default: return f(std::integral_constant<int, 32>{});
  }
}

template <class F>
static int with_ndof(int ndof, F&& f) {
  switch (ndof) {
    case 1: return f(std::integral_constant<int, 1>{});
    case 2: return f(std::integral_constant<int, 2>{});
    case 3: return f(std::integral_constant<int, 3>{});
  }
  return FOLGB_ERR_INVALID_ARGUMENT;
}

static int spmv_blocks(const folgb_plan* p, int G) {
  int64_t threads = p->N * (int64_t)G;
  int64_t blocks = (threads + 255) / 256;
  int64_t cap = (int64_t)num_sms() * 8;
  return (int)(blocks < cap ? blocks : cap);
}

__global__ void k_adam(float* __restrict__ x, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int64_t n, int* step, float lr, float b1, float b2, float eps) {
  // step counter read by every thread before block 0 increments it at the end
  const int t = *step + 1;
  const float bc1 = 1.f - powf(b1, (float)t), bc2 = 1.f - powf(b2, (float)t);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = fmaf(b1, m[i], (1.f - b1) * gi);
    const float vi = fmaf(b2, v[i], (1.f - b2) * gi * gi);
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / bc1, vh = vi / bc2;
    x[i] -= lr * mh / (sqrtf(vh) + eps);
  }
}

__global__ void k_step_inc(int* step) { *step += 1; }

}  // namespace folgb

using namespace folgb;

extern "C" int folgb_spmv(const folgb_plan* p, const float* vals, const float* x, float* y, void* stream) {
  if (!p || !vals || !x || !y) return FOLGB_ERR_INVALID_ARGUMENT;
  if (!p->has_csr) return FOLGB_ERR_NO_PATTERN;
  cudaStream_t s = (cudaStream_t)stream;
  return with_ndof(p->ndof, [&](auto nd) -> int {
    constexpr int NDOF = decltype(nd)::value;
    return with_group<NDOF>(p->maxdeg, [&](auto gw) -> int {
      constexpr int G = decltype(gw)::value;
      k_spmv<NDOF, G><<<spmv_blocks(p, G), 256, 0, s>>>(p->N, p->d_adj_ptr, p->d_adj, p->d_rowptr, vals, x, y);
      FOLGB_LAUNCH_CHECK();
      return (int)FOLGB_OK;
    });
  });
}

extern "C" int folgb_pcg(const folgb_plan* p, const float* vals, const float* dinv, const float* rhs, float* x,
                         double rtol, int32_t maxiter, int32_t check_every, int32_t* iterations, double* rel_residual,
                         void* workspace, size_t workspace_bytes, void* stream) {
  if (!p || !vals || !dinv || !rhs || !x || maxiter <= 0 || !(rtol >= 0.0)) return FOLGB_ERR_INVALID_ARGUMENT;
  if (!p->has_csr) return FOLGB_ERR_NO_PATTERN;
  PCGWork w;
  size_t need = layout_pcg(p, workspace, workspace_bytes, &w);
  if (!workspace || workspace_bytes < need) return FOLGB_ERR_WORKSPACE;
  if (check_every <= 0) check_every = 32;
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t n = (int64_t)p->ndof * p->N;
  int vb = (int)((n + 255) / 256);
  if (vb > kVecBlocks) vb = kVecBlocks;
  FOLGB_CUDA_TRY(cudaMemsetAsync(w.counters, 0, 4 * sizeof(unsigned), s));
  k_pcg_init<<<vb, 256, 0, s>>>(n, rhs, dinv, x, w.r, w.z, w.p0, w.part, w.counters, w.sc, rtol, maxiter);
  FOLGB_LAUNCH_CHECK();
  PCGScalars host{};
  int it = 0;
  float* pa = w.p0;
  float* pb = w.p1;
  int rc = with_ndof(p->ndof, [&](auto nd) -> int {
    constexpr int NDOF = decltype(nd)::value;
    return with_group<NDOF>(p->maxdeg, [&](auto gw) -> int {
      constexpr int G = decltype(gw)::value;
      const int sb = spmv_blocks(p, G);
      while (it < maxiter) {
        int chunk = check_every;
        if (chunk > maxiter - it) chunk = maxiter - it;
        for (int k = 0; k < chunk; ++k) {
          trace_begin(KID_PCG_SPMV, s);
          k_pcg_spmv<NDOF, G><<<sb, 256, 0, s>>>(p->N, p->d_adj_ptr, p->d_adj, p->d_rowptr, vals, w.z, pa, pb, w.q,
                                                  w.part, w.counters, w.sc);
          trace_end(KID_PCG_SPMV, s);
          trace_begin(KID_PCG_UPDATE, s);
          k_pcg_update<<<vb, 256, 0, s>>>(n, dinv, x, w.r, w.z, pb, w.q, w.part, w.counters, w.sc);
          trace_end(KID_PCG_UPDATE, s);
          float* t = pa;
          pa = pb;
          pb = t;
        }
        FOLGB_LAUNCH_CHECK();
        it += chunk;
        FOLGB_CUDA_TRY(cudaMemcpyAsync(&host, w.sc, sizeof(PCGScalars), cudaMemcpyDeviceToHost, s));
        FOLGB_CUDA_TRY(cudaStreamSynchronize(s));
        if (host.done) break;
      }
      return (int)FOLGB_OK;
    });
  });
  if (rc) return rc;
  if (iterations) *iterations = host.iters;
  if (rel_residual) *rel_residual = host.bnorm2 > 0 ? std::sqrt(host.rnorm2 / host.bnorm2) : 0.0;
  if (host.done == 3) return FOLGB_ERR_NAN;
  if (host.done != 1) return FOLGB_ERR_NOT_CONVERGED;
  return FOLGB_OK;
}

extern "C" int folgb_adam_step(float* params, const float* grads, float* m, float* v, int64_t n, int32_t* step,
                               float lr, float beta1, float beta2, float eps, void* stream) {
  if (!params || !grads || !m || !v || !step || n < 0) return FOLGB_ERR_INVALID_ARGUMENT;
  if (n == 0) return FOLGB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int blocks = (int)((n + 255) / 256);
  int cap = num_sms() * 8;
  if (blocks > cap) blocks = cap;
  k_adam<<<blocks, 256, 0, s>>>(params, grads, m, v, n, step, lr, beta1, beta2, eps);
  k_step_inc<<<1, 1, 0, s>>>(step);
  FOLGB_LAUNCH_CHECK();
  return FOLGB_OK;
}
