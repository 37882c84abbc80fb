// Krylov solvers on the plan's fixed CSR pattern (Jacobi-preconditioned CG and
// BiCGSTAB), SpMV, and the Adam update.  Replaces
// FiniteElementSolver.LinearSolve (fol/solvers/fe_solver.py:60-78; the
// reference's default is JAX BiCGSTAB, fe_solver.py:60-67).
//
// SpMV reads the canonical CSR values but indexes columns through the node
// adjacency (one column index per ndof x ndof block), so the index stream is
// 1/ndof^2 of a scalar CSR's.  One group of G lanes handles the ndof rows of
// a few consecutive nodes; lane k of the group owns the flat row positions
// k, k + G, ... (neighbour-major, component-minor), so value loads coalesce.
//
// Precision: matrix and Krylov vectors in fp32, every inner product and norm
// accumulated in fp64, the iterate x kept in fp64.  fp32 SpMV bounds how far
// the recurrence residual tracks the true one, so the solvers use reliable
// updates: when the recurrence residual has dropped 1e3 below the last true
// residual (or reached the tolerance) the host launches one fp64 SpMV that
// recomputes r = b - A x and restarts the recurrence from it.  Convergence is
// declared on that true residual only.
//
// Every iteration kernel returns at once when the device flags "done" or
// "replace" are set, so the host enqueues a chunk of iterations and reads
// the flags once per chunk.
#include <cmath>
#include <atomic>
#include <mutex>
#include <type_traits>

#include <cooperative_groups.h>

#include "folgb_internal.cuh"

using namespace folgb;

namespace folgb {

struct KScalars {
  double rho, bnorm2, rnorm2, rref2, tol2;
  double alpha, beta, omega;
  int iters, done, replace, maxiter, restart, breakdowns;
  int rounds;  // device-resident solve: executions of the loop body
  // which of the two direction buffers (p, and v for BiCGSTAB) holds the
  // current direction: flipped by the update kernel of every iteration that
  // ran, so iterations skipped after a replacement leave it in place
  int pcur;
};
// done: 1 converged (true residual), 2 maxiter, 3 non-finite, 4 repeated breakdown or divergence

// Outcome of a solve as the stream-ordered entry point reports it.
struct KReport {
  int32_t iterations, status;
  double rel_residual;
};

// Krylov vectors in VT (float, or double for ill-conditioned / indefinite
// systems such as the Neo-Hookean tangent); the iterate is always fp64.
template <class VT>
struct KWork {
  VT *r, *z, *p0, *p1, *q;   // PCG: r, z, p (two buffers), q = A p
  VT *rhat, *v0, *v1, *y, *t;  // BiCGSTAB extras
  double* x;                 // fp64 iterate
  double* part;              // [2][65536]
  unsigned* counters;        // [8]
  KScalars* sc;
  KReport* report;           // outcome of the synchronous entry points
};

constexpr int kVecBlocks = 1024;
// The PCG SpMV with fp32 vectors fits in 64 registers without spilling: 4
// blocks of 256 threads per SM (32 warps) keep more loads in flight than the
// 3 blocks an unconstrained build gives.  fp64 vectors, and the BiCGSTAB and
// true-residual kernels, would spill under that cap.
template <class VT>
constexpr int kSpmvMinBlocks = sizeof(VT) == sizeof(float) ? 4 : 1;
constexpr double kReplaceDrop2 = 1e-6;  // replace when |r|^2 <= 1e-6 |r_true|^2
constexpr int kMaxBreakdowns = 8;       // consecutive breakdown restarts before giving up
constexpr double kDiverge2 = 1e12;      // stop when |r_true|^2 > 1e12 |b|^2 (diverged)

template <class VT>
static size_t layout_krylov(const folgb_plan* p, void* base, size_t cap, KWork<VT>* w) {
  Bump bp(base, cap);
  const size_t n = (size_t)p->ndof * p->N;
  KWork<VT> t;
  t.r = bp.take<VT>(n);
  t.z = bp.take<VT>(n);
  t.p0 = bp.take<VT>(n);
  t.p1 = bp.take<VT>(n);
  t.q = bp.take<VT>(n);
  t.rhat = bp.take<VT>(n);
  t.v0 = bp.take<VT>(n);
  t.v1 = bp.take<VT>(n);
  t.y = bp.take<VT>(n);
  t.t = bp.take<VT>(n);
  t.x = bp.take<double>(n);
  t.part = bp.take<double>(2 * 65536);
  t.counters = bp.take<unsigned>(8);
  t.sc = bp.take<KScalars>(1);
  t.report = bp.take<KReport>(1);
  if (w) *w = t;
  return align_up(bp.off);
}

size_t pcg_workspace_bytes(const folgb_plan* p) { return layout_krylov<float>(p, nullptr, 0, nullptr); }
size_t krylov64_workspace_bytes(const folgb_plan* p) { return layout_krylov<double>(p, nullptr, 0, nullptr); }

__device__ __forceinline__ float vfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double vfma(double a, double b, double c) { return fma(a, b, c); }

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

// Row products over the node adjacency for U nodes at once.  The canonical
// CSR stores node n's ndof rows back to back, each ndof*deg(n) long and
// neighbour-major, so with a0 = adj_ptr[n] the value of row (n, i) at flat
// position w = ndof*j + l (neighbour j, component l) sits at
// ndof*ndof*a0 + i*ndof*deg + w: no rowptr read is needed.  A group of G
// lanes serves U consecutive nodes; lane k takes the flat positions
// w = k, k + G, ... of all ndof rows, so every value load of the group is
// contiguous (coalesced), and the loads of all U nodes are issued before any
// is used.
//
// The U*ndof per-lane partial sums are then reduced by halving: at each
// shuffle step a lane keeps half of its values (the upper half when its lane
// bit for that step is set) and adds the partner's copy of that half, so the
// group needs VP - 1 shuffles (VP = U*ndof rounded up to a power of two)
// instead of U*ndof*log2(G), and lane k ends up holding the row sum of value
// index k / (G / VP).  The row epilogues (vector updates, dot products) then
// run on U*ndof lanes in parallel instead of serially on one lane.
template <int NDOF>
struct RowsU {
  static constexpr int U = NDOF == 3 ? 5 : (NDOF == 2 ? 4 : 8);  // nodes per group per round
  static constexpr int V = U * NDOF;                              // rows per group per round
  static constexpr int VP = V <= 4 ? 4 : (V <= 8 ? 8 : 16);       // V rounded up to a power of two
};

template <int G, int C, int O, class T, int VP>
__device__ __forceinline__ void halving_reduce(T (&v)[VP], int lane) {
  if constexpr (C > 1) {
    const bool up = (lane & O) != 0;
#pragma unroll
    for (int k = 0; k < C / 2; ++k) {
      const T send = up ? v[k] : v[k + C / 2];
      const T keep = up ? v[k + C / 2] : v[k];
      v[k] = keep + __shfl_xor_sync(0xffffffffu, send, O, G);
    }
    halving_reduce<G, C / 2, O / 2>(v, lane);
  } else if constexpr (O >= 1) {
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], O, G);
    halving_reduce<G, 1, O / 2>(v, lane);
  }
}

// Returns true on the lane that owns a row of this round; then *sum is the
// row's product and *dof its index (node-major: ndof*node + component).
template <int NDOF, int G, class T, class Col>
__device__ __forceinline__ bool rows_multi(int64_t N, const int* __restrict__ adj_ptr, const int* __restrict__ adj,
                                           const float* __restrict__ vals, int maxdeg, int64_t base, int lane,
                                           Col col, T& sum, int64_t& dof) {
  constexpr int U = RowsU<NDOF>::U, V = RowsU<NDOF>::V, VP = RowsU<NDOF>::VP;
  static_assert(VP <= G, "lane group narrower than the rows it reduces");
  int a0[U], len[U];
  T acc[U][NDOF];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int64_t n = base + u;
    const bool act = n < N;
    a0[u] = act ? __ldg(adj_ptr + n) : 0;
    len[u] = act ? NDOF * (__ldg(adj_ptr + n + 1) - a0[u]) : 0;
#pragma unroll
    for (int i = 0; i < NDOF; ++i) acc[u][i] = T(0);
  }
  const int maxlen = NDOF * maxdeg;
  for (int w0 = 0; w0 < maxlen; w0 += G) {
    const int w = w0 + lane;
    const int j = w / NDOF, l = w - NDOF * j;
    int m[U];
    float v[U][NDOF];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const bool on = w < len[u];
      m[u] = on ? __ldg(adj + a0[u] + j) : 0;
      const float* vr = vals + (int64_t)NDOF * NDOF * a0[u] + w;
      // the values are read once per product: stream them evict-first so
      // they do not push the vectors and the adjacency out of L2
#pragma unroll
      for (int i = 0; i < NDOF; ++i) v[u][i] = on ? __ldcs(vr + (int64_t)i * len[u]) : 0.f;
    }
    T xv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) xv[u] = (w < len[u]) ? col((int64_t)NDOF * m[u] + l) : T(0);
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int i = 0; i < NDOF; ++i) acc[u][i] += (T)v[u][i] * xv[u];
  }
  T flat[VP];
#pragma unroll
  for (int k = 0; k < VP; ++k) flat[k] = k < V ? acc[k / NDOF][k % NDOF] : T(0);
  halving_reduce<G, VP, G / 2>(flat, lane);
  constexpr int kSub = G / VP;  // lanes sharing one value index
  const int idx = lane / kSub;
  sum = flat[0];
  dof = (int64_t)NDOF * base + idx;
  return (lane % kSub) == 0 && idx < V && dof < (int64_t)NDOF * N;
}

// Warp-uniform loop over node blocks: every lane runs the same number of
// rounds so the group shuffles always see the whole warp.
#define FOLGB_NODE_BLOCKS(NDOF, G)                                                               \
  constexpr int kU = RowsU<NDOF>::U;                                                             \
  const int lane = threadIdx.x % G;                                                              \
  const int64_t group = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;                    \
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;                                 \
  for (int64_t base = group * kU; __any_sync(0xffffffffu, base < N); base += ngroups * kU)

template <int NDOF, int G>
__global__ void __launch_bounds__(256) k_spmv(int64_t N, const int* __restrict__ adj_ptr, const int* __restrict__ adj,
                                              int maxdeg, const float* __restrict__ vals,
                                              const float* __restrict__ x, float* __restrict__ y) {
  FOLGB_NODE_BLOCKS(NDOF, G) {
    float sum;
    int64_t d;
    if (rows_multi<NDOF, G, float>(N, adj_ptr, adj, vals, maxdeg, base, lane,
                                   [&](int64_t k) { return __ldg(x + k); }, sum, d))
      y[d] = sum;
  }
}

// ---------------------------------------------------------------------------
// shared: fp64 true residual r = b - A x (reliable update / restart)
// ---------------------------------------------------------------------------
template <int NDOF, int G, bool BICG, class VT>
__global__ void __launch_bounds__(256) k_true_residual(int64_t N, const int* __restrict__ adj_ptr,
                                                       const int* __restrict__ adj, int maxdeg,
                                                       const float* __restrict__ vals, const float* __restrict__ b,
                                                       const float* __restrict__ dinv, const double* __restrict__ x,
                                                       VT* __restrict__ r, VT* __restrict__ z,
                                                       VT* __restrict__ rhat, double* part, unsigned* counters,
                                                       KScalars* sc) {
  __shared__ double sh[32];
  // runs only when an iteration kernel asked for it (in the device-resident
  // loop it is launched after every chunk)
  if (!sc->replace || sc->done) return;
  // Both solvers keep their search directions across a residual replacement
  // (restarting CG there would discard the conjugacy of the directions built
  // so far and slow the convergence of the error); only a breakdown
  // (replace == 2) restarts them: BiCGSTAB from rhat = r, CG from p = z.
  const bool restart = sc->replace == 2;
  VT rzf = VT(0);
  double rr = 0.0;
  FOLGB_NODE_BLOCKS(NDOF, G) {
    double sum;
    int64_t d;
    if (rows_multi<NDOF, G, double>(N, adj_ptr, adj, vals, maxdeg, base, lane, [&](int64_t k) { return x[k]; },
                                    sum, d)) {
      const double ri = (double)b[d] - sum;
      const VT rf = (VT)ri;
      r[d] = rf;
      if (!BICG) {
        const VT zf = (VT)dinv[d] * rf;
        z[d] = zf;
        rzf = vfma(rf, zf, rzf);
      } else if (BICG && restart) {
        rhat[d] = rf;
        rzf = vfma(rf, rf, rzf);
      } else {
        rzf = vfma(rhat[d], rf, rzf);
      }
      rr = fma(ri, ri, rr);
    }
  }
  double s1 = block_sum_d((double)rzf, sh);
  double s2 = block_sum_d(rr, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = s1;
    part[gridDim.x + blockIdx.x] = s2;
  }
  if (!last_block(&counters[3])) return;
  double RZ = sum_partials(part, gridDim.x, sh);
  double RR = sum_partials(part + gridDim.x, gridDim.x, sh);
  if (threadIdx.x == 0) {
    sc->rnorm2 = RR;
    sc->rref2 = RR;
    sc->replace = 0;
    if (BICG) {
      if (restart) sc->restart = 1;
    } else if (restart || !(sc->rho > 0.0) || sc->beta == 0.0) {
      sc->beta = 0.0;  // breakdown: restart the search direction, p = z
    } else {
      // the next direction p = z + beta p_old with beta = (r . z) / rho_old
      // of the replaced residual; the update kernel left beta = rz / rho_old
      // and rho = rz of the recurrence residual, so rho_old = rho / beta
      sc->beta = RZ * sc->beta / sc->rho;
    }
    sc->rho = RZ;  // PCG: r . z;  BiCGSTAB: rhat . r
    if (!isfinite(RR)) sc->done = 3;
    else if (RR <= sc->tol2) sc->done = 1;
    else if (RR > kDiverge2 * sc->bnorm2) sc->done = 4;
    counters[3] = 0u;
  }
}

__global__ void k_to_float(int64_t n, const double* __restrict__ x, float* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)x[i];
}

// ---------------------------------------------------------------------------
// Jacobi PCG
// ---------------------------------------------------------------------------
template <class VT>
__global__ void k_pcg_init(int64_t n, const float* __restrict__ b, const float* __restrict__ dinv,
                           double* __restrict__ x, VT* __restrict__ r, VT* __restrict__ z, VT* __restrict__ p0,
                           double* part, unsigned* counters, KScalars* sc, double rtol, int maxiter) {
  __shared__ double sh[32];
  double rz = 0.0, bb = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float bi = b[i];
    float zi = dinv[i] * bi;
    x[i] = 0.0;
    r[i] = bi;
    z[i] = zi;
    p0[i] = VT(0);
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
    sc->rref2 = BB;
    sc->tol2 = rtol * rtol * BB;
    sc->alpha = sc->beta = 0.0;
    sc->omega = 1.0;
    sc->iters = 0;
    sc->maxiter = maxiter;
    sc->replace = 0;
    sc->restart = 0;
    sc->breakdowns = 0;
    sc->rounds = 0;
    sc->pcur = 0;
    sc->done = (BB == 0.0 || !isfinite(BB)) ? (BB == 0.0 ? 1 : 3) : 0;
    counters[0] = 0u;
  }
}

template <int NDOF, int G, class VT>
__global__ void __launch_bounds__(256, kSpmvMinBlocks<VT>) k_pcg_spmv(int64_t N, const int* __restrict__ adj_ptr,
                                                  const int* __restrict__ adj, int maxdeg,
                                                  const float* __restrict__ vals, const VT* __restrict__ z,
                                                  VT* pbuf0, VT* pbuf1, VT* __restrict__ q, double* part,
                                                  unsigned* counters, KScalars* sc) {
  __shared__ double sh[32];
  if (sc->done || sc->replace) return;
  const VT* __restrict__ pold = sc->pcur ? pbuf1 : pbuf0;
  VT* __restrict__ pnew = sc->pcur ? pbuf0 : pbuf1;
  const VT beta = (VT)sc->beta;
  VT dot = VT(0);  // this lane's rows only (a handful); fp64 from the block sum on
  FOLGB_NODE_BLOCKS(NDOF, G) {
    VT sum;
    int64_t d;
    if (rows_multi<NDOF, G, VT>(N, adj_ptr, adj, vals, maxdeg, base, lane,
                                [&](int64_t k) { return vfma(beta, __ldg(pold + k), __ldg(z + k)); }, sum, d)) {
      const VT pn = vfma(beta, pold[d], z[d]);
      pnew[d] = pn;
      q[d] = sum;
      dot = vfma(pn, sum, dot);
    }
  }
  double s = block_sum_d((double)dot, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  if (!last_block(&counters[1])) return;
  double PQ = sum_partials(part, gridDim.x, sh);
  if (threadIdx.x == 0) {
    if (!(PQ > 0.0) || !isfinite(PQ)) {
      // breakdown: restart from the true residual; give up if it repeats
      sc->alpha = 0.0;
      sc->breakdowns += 1;
      if (!isfinite(PQ)) sc->done = 3;
      else if (sc->breakdowns > kMaxBreakdowns) sc->done = 4;
      else sc->replace = 2;
    } else {
      sc->alpha = sc->rho / PQ;
    }
    counters[1] = 0u;
  }
}

template <class VT>
__global__ void __launch_bounds__(256) k_pcg_update(int64_t n, const float* __restrict__ dinv,
                                                    double* __restrict__ x, VT* __restrict__ r, VT* __restrict__ z,
                                                    const VT* pbuf0, const VT* pbuf1, const VT* __restrict__ q,
                                                    double* part, unsigned* counters, KScalars* sc) {
  __shared__ double sh[32];
  if (sc->done || sc->replace) return;
  const VT* __restrict__ p = sc->pcur ? pbuf0 : pbuf1;  // the direction the SpMV just wrote
  const double alpha = sc->alpha;
  const VT af = (VT)alpha;
  VT rz = VT(0), rr = VT(0);  // per-thread partials over a few entries
  // four independent entries per trip: their loads are in flight together
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {
    double xv[4];
    VT pv[4], qv[4], rv[4];
    float dv[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int64_t j = i + k * stride;
      xv[k] = x[j];
      pv[k] = p[j];
      qv[k] = q[j];
      rv[k] = r[j];
      dv[k] = dinv[j];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int64_t j = i + k * stride;
      x[j] = fma(alpha, (double)pv[k], xv[k]);
      const VT ri = vfma(-af, qv[k], rv[k]);
      r[j] = ri;
      const VT zi = (VT)dv[k] * ri;
      z[j] = zi;
      rz = vfma(ri, zi, rz);
      rr = vfma(ri, ri, rr);
    }
  }
  for (; i < n; i += stride) {
    x[i] = fma(alpha, (double)p[i], x[i]);
    const VT ri = vfma(-af, q[i], r[i]);
    r[i] = ri;
    const VT zi = (VT)dinv[i] * ri;
    z[i] = zi;
    rz = vfma(ri, zi, rz);
    rr = vfma(ri, ri, rr);
  }
  double s1 = block_sum_d((double)rz, sh);
  double s2 = block_sum_d((double)rr, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = s1;
    part[gridDim.x + blockIdx.x] = s2;
  }
  if (!last_block(&counters[2])) return;
  double RZ = sum_partials(part, gridDim.x, sh);
  double RR = sum_partials(part + gridDim.x, gridDim.x, sh);
  if (threadIdx.x == 0) {
    sc->beta = RZ / sc->rho;
    sc->rho = RZ;
    sc->rnorm2 = RR;
    sc->iters += 1;
    sc->breakdowns = 0;
    sc->pcur ^= 1;
    if (!isfinite(RR)) sc->done = 3;
    else if (RR <= sc->tol2 || RR <= kReplaceDrop2 * sc->rref2 || RR > kDiverge2 * sc->bnorm2) sc->replace = 1;
    if (!sc->done && sc->iters >= sc->maxiter) sc->replace = 1;
    counters[2] = 0u;
  }
}

// ---------------------------------------------------------------------------
// Jacobi BiCGSTAB (right preconditioned): y = D^-1 p, z = D^-1 s,
// x += alpha y + omega z.  Three kernels per iteration.
// ---------------------------------------------------------------------------
template <class VT>
__global__ void k_bicg_init(int64_t n, const float* __restrict__ b, double* __restrict__ x, VT* __restrict__ r,
                            VT* __restrict__ rhat, double* part, unsigned* counters, KScalars* sc, double rtol,
                            int maxiter) {
  __shared__ double sh[32];
  double bb = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float bi = b[i];
    x[i] = 0.0;
    r[i] = bi;
    rhat[i] = bi;
    bb += (double)bi * (double)bi;
  }
  double s2 = block_sum_d(bb, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s2;
  if (!last_block(&counters[0])) return;
  double BB = sum_partials(part, gridDim.x, sh);
  if (threadIdx.x == 0) {
    sc->rho = BB;
    sc->bnorm2 = BB;
    sc->rnorm2 = BB;
    sc->rref2 = BB;
    sc->tol2 = rtol * rtol * BB;
    sc->alpha = sc->omega = 1.0;
    sc->beta = 0.0;
    sc->iters = 0;
    sc->maxiter = maxiter;
    sc->replace = 0;
    sc->restart = 1;
    sc->breakdowns = 0;
    sc->rounds = 0;
    sc->pcur = 0;
    sc->done = (BB == 0.0 || !isfinite(BB)) ? (BB == 0.0 ? 1 : 3) : 0;
    counters[0] = 0u;
  }
}

// p_new = r + beta (p_old - omega v_old) (p_new = r on restart), y = D^-1 p_new,
// v_new = A y; alpha = rho / (rhat . v_new)
template <int NDOF, int G, class VT>
__global__ void __launch_bounds__(256) k_bicg_p_spmv(int64_t N, const int* __restrict__ adj_ptr,
                                                     const int* __restrict__ adj, int maxdeg,
                                                     const float* __restrict__ vals, const float* __restrict__ dinv,
                                                     const VT* __restrict__ r, const VT* __restrict__ rhat,
                                                     VT* pbuf0, VT* pbuf1, VT* vbuf0, VT* vbuf1,
                                                     VT* __restrict__ y, double* part, unsigned* counters,
                                                     KScalars* sc) {
  __shared__ double sh[32];
  if (sc->done || sc->replace) return;
  const int c = sc->pcur;
  const VT* __restrict__ pold = c ? pbuf1 : pbuf0;
  const VT* __restrict__ vold = c ? vbuf1 : vbuf0;
  VT* __restrict__ pnew = c ? pbuf0 : pbuf1;
  VT* __restrict__ vnew = c ? vbuf0 : vbuf1;
  const bool rs = sc->restart != 0;
  const VT beta = rs ? VT(0) : (VT)sc->beta;
  const VT omega = rs ? VT(0) : (VT)sc->omega;
  auto pval = [&](int64_t d) -> VT {
    return rs ? __ldg(r + d) : vfma(beta, vfma(-omega, __ldg(vold + d), __ldg(pold + d)), __ldg(r + d));
  };
  VT dot = VT(0);
  FOLGB_NODE_BLOCKS(NDOF, G) {
    VT sum;
    int64_t d;
    if (rows_multi<NDOF, G, VT>(N, adj_ptr, adj, vals, maxdeg, base, lane,
                                [&](int64_t k) { return (VT)__ldg(dinv + k) * pval(k); }, sum, d)) {
      const VT pn = pval(d);
      pnew[d] = pn;
      y[d] = (VT)dinv[d] * pn;
      vnew[d] = sum;
      dot = vfma(rhat[d], sum, dot);
    }
  }
  double s = block_sum_d((double)dot, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  if (!last_block(&counters[1])) return;
  double RV = sum_partials(part, gridDim.x, sh);
  if (threadIdx.x == 0) {
    sc->restart = 0;
    if (RV == 0.0 || !isfinite(RV)) {
      sc->breakdowns += 1;
      if (!isfinite(RV)) sc->done = 3;
      else if (sc->breakdowns > kMaxBreakdowns) sc->done = 4;
      else sc->replace = 2;
    } else {
      sc->alpha = sc->rho / RV;
    }
    counters[1] = 0u;
  }
}

// s = r - alpha v_new, z = D^-1 s, t = A z; omega = (t . s) / (t . t)
template <int NDOF, int G, class VT>
__global__ void __launch_bounds__(256) k_bicg_s_spmv(int64_t N, const int* __restrict__ adj_ptr,
                                                     const int* __restrict__ adj, int maxdeg,
                                                     const float* __restrict__ vals, const float* __restrict__ dinv,
                                                     const VT* __restrict__ r, const VT* vbuf0, const VT* vbuf1,
                                                     VT* __restrict__ z, VT* __restrict__ t, double* part,
                                                     unsigned* counters, KScalars* sc) {
  __shared__ double sh[32];
  if (sc->done || sc->replace) return;
  const VT* __restrict__ vnew = sc->pcur ? vbuf0 : vbuf1;
  const VT af = (VT)sc->alpha;
  auto sval = [&](int64_t d) -> VT { return vfma(-af, __ldg(vnew + d), __ldg(r + d)); };
  VT ts = VT(0), tt = VT(0);
  FOLGB_NODE_BLOCKS(NDOF, G) {
    VT sum;
    int64_t d;
    if (rows_multi<NDOF, G, VT>(N, adj_ptr, adj, vals, maxdeg, base, lane,
                                [&](int64_t k) { return (VT)__ldg(dinv + k) * sval(k); }, sum, d)) {
      const VT sv = sval(d);
      z[d] = (VT)dinv[d] * sv;
      t[d] = sum;
      ts = vfma(sum, sv, ts);
      tt = vfma(sum, sum, tt);
    }
  }
  double s1 = block_sum_d((double)ts, sh);
  double s2 = block_sum_d((double)tt, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = s1;
    part[gridDim.x + blockIdx.x] = s2;
  }
  if (!last_block(&counters[4])) return;
  double TS = sum_partials(part, gridDim.x, sh);
  double TT = sum_partials(part + gridDim.x, gridDim.x, sh);
  if (threadIdx.x == 0) {
    sc->omega = (TT > 0.0 && isfinite(TT)) ? TS / TT : 0.0;
    counters[4] = 0u;
  }
}

template <class VT>
__global__ void __launch_bounds__(256) k_bicg_update(int64_t n, double* __restrict__ x, VT* __restrict__ r,
                                                     const VT* __restrict__ rhat, const VT* vbuf0, const VT* vbuf1,
                                                     const VT* __restrict__ y, const VT* __restrict__ z,
                                                     const VT* __restrict__ t, double* part, unsigned* counters,
                                                     KScalars* sc) {
  __shared__ double sh[32];
  if (sc->done || sc->replace) return;
  const VT* __restrict__ vnew = sc->pcur ? vbuf0 : vbuf1;
  const double alpha = sc->alpha, omega = sc->omega;
  const VT af = (VT)alpha, of = (VT)omega;
  VT rhr = VT(0), rr = VT(0);  // per-thread partials over a few entries
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const VT s = vfma(-af, vnew[i], r[i]);
    x[i] = fma(omega, (double)z[i], fma(alpha, (double)y[i], x[i]));
    const VT ri = vfma(-of, t[i], s);
    r[i] = ri;
    rhr = vfma(rhat[i], ri, rhr);
    rr = vfma(ri, ri, rr);
  }
  double s1 = block_sum_d((double)rhr, sh);
  double s2 = block_sum_d((double)rr, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = s1;
    part[gridDim.x + blockIdx.x] = s2;
  }
  if (!last_block(&counters[2])) return;
  double RH = sum_partials(part, gridDim.x, sh);
  double RR = sum_partials(part + gridDim.x, gridDim.x, sh);
  if (threadIdx.x == 0) {
    const double rho_old = sc->rho;
    sc->beta = (omega != 0.0 && rho_old != 0.0) ? (RH / rho_old) * (alpha / omega) : 0.0;
    sc->rho = RH;
    sc->rnorm2 = RR;
    sc->iters += 1;
    sc->breakdowns = 0;
    sc->pcur ^= 1;
    if (!isfinite(RR)) sc->done = 3;
    else if (RH == 0.0 || omega == 0.0) sc->replace = 2;  // breakdown: restart
    else if (RR <= sc->tol2 || RR <= kReplaceDrop2 * sc->rref2 || RR > kDiverge2 * sc->bnorm2) sc->replace = 1;
    if (!sc->done && sc->iters >= sc->maxiter) sc->replace = 1;
    counters[2] = 0u;
  }
}

// Loop control of the device-resident solve (a CUDA-graph WHILE node whose
// body is one chunk of iterations + the true-residual kernel + this kernel):
// the same exits as the host loop, and a hard cap on body executions so the
// loop always ends.
__global__ void k_krylov_continue(KScalars* sc, cudaGraphConditionalHandle loop, int maxiter, int max_rounds) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (!sc->done && !sc->replace && sc->iters >= maxiter) sc->done = 2;
  sc->rounds += 1;
  if (!sc->done && sc->rounds >= max_rounds) sc->done = 2;
  cudaGraphSetConditional(loop, sc->done ? 0u : 1u);
}

__global__ void k_arm_conditional(cudaGraphConditionalHandle h) {
  if (threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(h, 1u);
}

template <int NDOF>
static int group_width(int maxdeg) {
  int g = 1;
  while (g < NDOF * maxdeg && g < 32) g <<= 1;
  return g < RowsU<NDOF>::VP ? RowsU<NDOF>::VP : g;
}

template <int NDOF, class F>
static int with_group(int maxdeg, F&& f) {
  constexpr int VP = RowsU<NDOF>::VP;  // group_width never returns less
  switch (group_width<NDOF>(maxdeg)) {
    case 4:
      if constexpr (VP <= 4) return f(std::integral_constant<int, 4>{});
      break;
    case 8:
      if constexpr (VP <= 8) return f(std::integral_constant<int, 8>{});
      break;
    case 16:
      if constexpr (VP <= 16) return f(std::integral_constant<int, 16>{});
      break;
    default:
      break;
  }
  return f(std::integral_constant<int, 32>{});
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

template <int NDOF>
static int spmv_blocks(const folgb_plan* p, int G) {
  constexpr int U = RowsU<NDOF>::U;
  int64_t threads = ((p->N + U - 1) / U) * (int64_t)G;
  int64_t blocks = (threads + 255) / 256;
  int64_t cap = (int64_t)num_sms() * 8;
  return (int)(blocks < cap ? blocks : cap);
}

// One Adam update (optax.adam): the bias corrections enter as the reciprocals
// of 1 - beta^t, formed once per launch.
struct AdamCoef {
  float lr, b1, b2, eps, rb1, rb2;
};

__device__ __forceinline__ void adam_one(const AdamCoef& c, float& x, float g, float& m, float& v) {
  m = fmaf(c.b1, m, (1.f - c.b1) * g);
  v = fmaf(c.b2, v, (1.f - c.b2) * g * g);
  x -= c.lr * (m * c.rb1) / (sqrtf(v * c.rb2) + c.eps);
}

// 16-byte loads and stores when all four arrays are 16-byte aligned (four
// parameters per trip), plain ones otherwise and for the last n mod 4.
__global__ void k_adam(float* __restrict__ x, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int64_t n, const int* step, float lr, float b1, float b2, float eps) {
  const int t = *step + 1;
  const AdamCoef c{lr, b1, b2, eps, 1.f / (1.f - powf(b1, (float)t)), 1.f / (1.f - powf(b2, (float)t))};
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  const bool vec = ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(g) | reinterpret_cast<uintptr_t>(m) |
                     reinterpret_cast<uintptr_t>(v)) & 15u) == 0;
  int64_t done = 0;
  if (vec) {
    const int64_t n4 = n >> 2;
    float4* x4 = reinterpret_cast<float4*>(x);
    const float4* g4 = reinterpret_cast<const float4*>(g);
    float4* m4 = reinterpret_cast<float4*>(m);
    float4* v4 = reinterpret_cast<float4*>(v);
    for (int64_t i = tid; i < n4; i += stride) {
      float4 xv = x4[i], mv = m4[i], vv = v4[i];
      const float4 gv = g4[i];
      adam_one(c, xv.x, gv.x, mv.x, vv.x);
      adam_one(c, xv.y, gv.y, mv.y, vv.y);
      adam_one(c, xv.z, gv.z, mv.z, vv.z);
      adam_one(c, xv.w, gv.w, mv.w, vv.w);
      x4[i] = xv;
      m4[i] = mv;
      v4[i] = vv;
    }
    done = n4 << 2;
  }
  for (int64_t i = done + tid; i < n; i += stride) {
    float xi = x[i], mi = m[i], vi = v[i];
    adam_one(c, xi, g[i], mi, vi);
    x[i] = xi;
    m[i] = mi;
    v[i] = vi;
  }
}

__global__ void k_step_inc(int* step) { *step += 1; }

enum { SOLVER_CG = 0, SOLVER_BICGSTAB = 1 };

// Engine of large fp32 CG solves (folgb_krylov_set_engine): the grid-resident
// CG by default.
static std::atomic<int> g_krylov_engine{FOLGB_KRYLOV_ENGINE_GRID};
static int krylov_engine() { return g_krylov_engine.load(); }

// ---------------------------------------------------------------------------
// Cluster-resident solver for small systems: the whole solve is ONE launch of
// one thread-block cluster (kClusterCTAs CTAs on as many SMs).  Each CTA owns a
// contiguous range of nodes (rows); vectors live in global memory (L2), the
// iteration's phases are separated by hardware cluster barriers, and every
// reduction is done by each CTA posting its block sum in shared memory and
// every CTA adding all CTAs' sums in rank order over distributed shared
// memory -- so all CTAs hold bit-identical scalars and take the same branch.
// No host round trip, no kernel boundary, no spin-wait.  Same algorithm,
// precision scheme and exits as the multi-kernel solver above.
// ---------------------------------------------------------------------------
constexpr int kClusterCTAs = 16;          // non-portable size (opt-in); 8, the portable one, as fallback
constexpr int kClusterThreads = 512;
constexpr int64_t kClusterMaxDofs = 16384;  // measured crossover: ~2x faster at 2.6k-6.6k dofs, slower at 47k

template <class VT>
struct ClusterArgs {
  int64_t N;
  const int* adj_ptr;
  const int* adj;
  int maxdeg;
  const float* vals;
  const float* dinv;
  const float* b;
  VT *r, *z, *p, *q, *rhat, *v, *y, *t;
  double* x;
  float* xout;
  KScalars* sc;
  double rtol;
  int maxiter;
};

// sum of K doubles over the cluster; every thread of every CTA gets the same
// totals (block sums added in rank order)
template <int K>
__device__ __forceinline__ void cluster_sum(double (&v)[K], double* sh, double (*slot)[4], int& parity) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const double s = block_sum_d(v[k], sh);
    if (threadIdx.x == 0) slot[parity][k] = s;
  }
  cluster.sync();
  // lane r of every warp fetches rank r's sums (one remote latency, not nr),
  // then a fixed shuffle tree adds them: the same order in every warp and CTA
  const int nr = (int)cluster.num_blocks(), lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double tot = lane < nr ? cluster.map_shared_rank(&slot[parity][0], lane)[k] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
    v[k] = tot;
  }
  parity ^= 1;
}

// rows of this CTA's node range [n0, n1): epi(dof, row sum) on the owner lanes
template <int NDOF, int G, class T, class VT, class Col, class Epi>
__device__ __forceinline__ void cta_rows(const ClusterArgs<VT>& A, int64_t n0, int64_t n1, Col col, Epi epi) {
  constexpr int U = RowsU<NDOF>::U;
  const int lane = threadIdx.x % G;
  const int64_t group = threadIdx.x / G, ngroups = blockDim.x / G;
  for (int64_t base = n0 + group * U; __any_sync(0xffffffffu, base < n1); base += ngroups * U) {
    T sum;
    int64_t d;
    if (rows_multi<NDOF, G, T>(n1, A.adj_ptr, A.adj, A.vals, A.maxdeg, base, lane, col, sum, d)) epi(d, sum);
  }
}

template <int NDOF, int G, class VT, bool BICG>
__global__ void __launch_bounds__(kClusterThreads, 1) k_krylov_cluster(const ClusterArgs<VT> A) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  __shared__ double sh[32];
  __shared__ double slot[2][4];
  int parity = 0;
  const int rank = (int)cluster.block_rank(), nr = (int)cluster.num_blocks();
  const int64_t n0 = A.N * rank / nr, n1 = A.N * (rank + 1) / nr;
  const int64_t d0 = NDOF * n0, d1 = NDOF * n1;
  const int64_t tid = threadIdx.x, nth = blockDim.x;
  // ---- init: x = 0, r = b (BiCGSTAB: rhat = r; CG: z = D^-1 r, p = 0)
  double red[2] = {0.0, 0.0};
  for (int64_t d = d0 + tid; d < d1; d += nth) {
    const float bi = A.b[d];
    A.x[d] = 0.0;
    A.r[d] = (VT)bi;
    if (BICG) {
      A.rhat[d] = (VT)bi;
    } else {
      const VT zi = (VT)A.dinv[d] * (VT)bi;
      A.z[d] = zi;
      A.p[d] = VT(0);
      red[1] += (double)bi * (double)zi;
    }
    red[0] += (double)bi * (double)bi;
  }
  cluster_sum<2>(red, sh, slot, parity);
  const double bb = red[0];
  const double tol2 = A.rtol * A.rtol * bb;
  double rho = BICG ? bb : red[1], rref2 = bb, rnorm2 = bb;
  double alpha = 1.0, beta = 0.0, omega = 1.0;
  int done = (bb == 0.0) ? 1 : (!isfinite(bb) ? 3 : 0);
  int iters = 0, breakdowns = 0, replace = 0;
  bool restart = true;
  while (!done) {
    if (!replace) {
      if constexpr (BICG) {
        // A: p = r + beta (p - omega v) (p = r on restart), y = D^-1 p
        const VT vb = (VT)beta, vo = (VT)omega;
        for (int64_t d = d0 + tid; d < d1; d += nth) {
          const VT pn = restart ? A.r[d] : vfma(vb, vfma(-vo, A.v[d], A.p[d]), A.r[d]);
          A.p[d] = pn;
          A.y[d] = (VT)A.dinv[d] * pn;
        }
        cluster.sync();
        // B: v = A y, rhat . v
        double dv[1] = {0.0};
        cta_rows<NDOF, G, VT>(A, n0, n1, [&](int64_t k) { return A.y[k]; }, [&](int64_t d, VT sum) {
          A.v[d] = sum;
          dv[0] += (double)A.rhat[d] * (double)sum;
        });
        cluster_sum<1>(dv, sh, slot, parity);
        const double RV = dv[0];
        restart = false;
        if (RV == 0.0 || !isfinite(RV)) {
          ++breakdowns;
          if (!isfinite(RV)) done = 3;
          else if (breakdowns > kMaxBreakdowns) done = 4;
          else replace = 2;
          continue;
        }
        alpha = rho / RV;
        // C: s = r - alpha v (kept in q), z = D^-1 s
        const VT va = (VT)alpha;
        for (int64_t d = d0 + tid; d < d1; d += nth) {
          const VT sv = vfma(-va, A.v[d], A.r[d]);
          A.q[d] = sv;
          A.z[d] = (VT)A.dinv[d] * sv;
        }
        cluster.sync();
        // D: t = A z, t . s, t . t
        double dt[2] = {0.0, 0.0};
        cta_rows<NDOF, G, VT>(A, n0, n1, [&](int64_t k) { return A.z[k]; }, [&](int64_t d, VT sum) {
          A.t[d] = sum;
          dt[0] += (double)sum * (double)A.q[d];
          dt[1] += (double)sum * (double)sum;
        });
        cluster_sum<2>(dt, sh, slot, parity);
        omega = (dt[1] > 0.0 && isfinite(dt[1])) ? dt[0] / dt[1] : 0.0;
        // E: x += alpha y + omega z, r = s - omega t, rhat . r, r . r
        const VT vom = (VT)omega;
        double de[2] = {0.0, 0.0};
        for (int64_t d = d0 + tid; d < d1; d += nth) {
          A.x[d] = fma(omega, (double)A.z[d], fma(alpha, (double)A.y[d], A.x[d]));
          const VT ri = vfma(-vom, A.t[d], A.q[d]);
          A.r[d] = ri;
          de[0] += (double)A.rhat[d] * (double)ri;
          de[1] += (double)ri * (double)ri;
        }
        cluster_sum<2>(de, sh, slot, parity);
        const double RH = de[0], RR = de[1];
        beta = (omega != 0.0 && rho != 0.0) ? (RH / rho) * (alpha / omega) : 0.0;
        rho = RH;
        rnorm2 = RR;
        ++iters;
        breakdowns = 0;
        if (!isfinite(RR)) done = 3;
        else if (RH == 0.0 || omega == 0.0) replace = 2;
        else if (RR <= tol2 || RR <= kReplaceDrop2 * rref2 || RR > kDiverge2 * bb) replace = 1;
        if (!done && iters >= A.maxiter) replace = replace ? replace : 1;
      } else {
        // A: p = z + beta p
        const VT vb = (VT)beta;
        for (int64_t d = d0 + tid; d < d1; d += nth) A.p[d] = vfma(vb, A.p[d], A.z[d]);
        cluster.sync();
        // B: q = A p, p . q
        double dq[1] = {0.0};
        cta_rows<NDOF, G, VT>(A, n0, n1, [&](int64_t k) { return A.p[k]; }, [&](int64_t d, VT sum) {
          A.q[d] = sum;
          dq[0] += (double)A.p[d] * (double)sum;
        });
        cluster_sum<1>(dq, sh, slot, parity);
        const double PQ = dq[0];
        if (!(PQ > 0.0) || !isfinite(PQ)) {
          ++breakdowns;
          if (!isfinite(PQ)) done = 3;
          else if (breakdowns > kMaxBreakdowns) done = 4;
          else replace = 2;
          continue;
        }
        alpha = rho / PQ;
        // C: x += alpha p, r -= alpha q, z = D^-1 r, r . z, r . r
        const VT va = (VT)alpha;
        double dc[2] = {0.0, 0.0};
        for (int64_t d = d0 + tid; d < d1; d += nth) {
          A.x[d] = fma(alpha, (double)A.p[d], A.x[d]);
          const VT ri = vfma(-va, A.q[d], A.r[d]);
          A.r[d] = ri;
          const VT zi = (VT)A.dinv[d] * ri;
          A.z[d] = zi;
          dc[0] += (double)ri * (double)zi;
          dc[1] += (double)ri * (double)ri;
        }
        cluster_sum<2>(dc, sh, slot, parity);
        const double RZ = dc[0], RR = dc[1];
        beta = RZ / rho;
        rho = RZ;
        rnorm2 = RR;
        ++iters;
        breakdowns = 0;
        if (!isfinite(RR)) done = 3;
        else if (RR <= tol2 || RR <= kReplaceDrop2 * rref2 || RR > kDiverge2 * bb) replace = 1;
        if (!done && iters >= A.maxiter) replace = replace ? replace : 1;
      }
      if (done || !replace) continue;
    }
    // reliable update: r = b - A x in fp64 (x of every CTA is visible: the
    // last cluster sum ordered it); a breakdown (replace == 2) also restarts
    // BiCGSTAB's shadow residual
    const bool fresh = BICG && replace == 2;
    double dr[2] = {0.0, 0.0};
    cta_rows<NDOF, G, double>(A, n0, n1, [&](int64_t k) { return A.x[k]; }, [&](int64_t d, double sum) {
      const double ri = (double)A.b[d] - sum;
      const VT rv = (VT)ri;
      A.r[d] = rv;
      if (!BICG) {
        const VT zi = (VT)A.dinv[d] * rv;
        A.z[d] = zi;
        dr[0] += (double)rv * (double)zi;
      } else if (fresh) {
        A.rhat[d] = rv;
        dr[0] += (double)rv * (double)rv;
      } else {
        dr[0] += (double)A.rhat[d] * (double)rv;
      }
      dr[1] += ri * ri;
    });
    cluster_sum<2>(dr, sh, slot, parity);
    // CG keeps its direction across a replacement (beta = (r . z) / rho_old
    // of the replaced residual, rho_old = rho / beta); a breakdown restarts it
    if (!BICG) beta = (replace == 2 || !(rho > 0.0) || beta == 0.0) ? 0.0 : dr[0] * beta / rho;
    rho = dr[0];
    rref2 = rnorm2 = dr[1];
    if (fresh) restart = true;
    replace = 0;
    if (!isfinite(dr[1])) done = 3;
    else if (dr[1] <= tol2) done = 1;
    else if (dr[1] > kDiverge2 * bb) done = 4;
    else if (iters >= A.maxiter) done = 2;
  }
  for (int64_t d = d0 + tid; d < d1; d += nth) A.xout[d] = (float)A.x[d];
  if (rank == 0 && threadIdx.x == 0) {
    A.sc->iters = iters;
    A.sc->done = done;
    A.sc->rnorm2 = rnorm2;
    A.sc->bnorm2 = bb;
  }
}

// one launch of the cluster solver; returns false if the launch was refused
// (the caller then uses the multi-kernel path)
template <int NDOF, int G, class VT>
static bool launch_cluster_solver(int solver, const ClusterArgs<VT>& A, cudaStream_t s) {
  auto kernel = solver == SOLVER_CG ? k_krylov_cluster<NDOF, G, VT, false> : k_krylov_cluster<NDOF, G, VT, true>;
  for (int ctas : {kClusterCTAs, 8}) {
    if (ctas > 8 && cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = ctas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, kernel, &cfg) != cudaSuccess || nclusters < 1) {
      cudaGetLastError();
      continue;
    }
    if (cudaLaunchKernelEx(&cfg, kernel, A) == cudaSuccess) return true;
    cudaGetLastError();
  }
  return false;
}

// ---------------------------------------------------------------------------
// Grid-resident Jacobi-PCG for large systems: the whole solve is ONE
// cooperative launch (every block resident), each block owning a contiguous
// node range; the phases of an iteration are separated by grid barriers on a
// global counter (bounded waits), and every reduction is each block posting its
// block sums and every block adding all posts in block order, so all blocks
// hold bit-identical scalars.  Per iteration two barriers:
//   B: p_new = z + beta p_old formed on the fly for the SpMV's columns (p is
//      double-buffered, so no block overwrites what another still reads),
//      q = A p_new, p . q                                      -> barrier, alpha
//   C: x += alpha p_new (fp64), r -= alpha q, z = D^-1 r, r . z, r . r
//                                                              -> barrier, beta
// Reliable updates as the multi-kernel solver (true residual in fp64, the
// direction kept unless a breakdown restarts it).  Vectors written during the
// solve are read through L2 (ld.global.cg), never a stale L1 line.
// ---------------------------------------------------------------------------
constexpr int kGridThreads = 512;

template <class VT>
struct GridArgs {
  int64_t N;
  const int* adj_ptr;
  const int* adj;
  int maxdeg;
  const float* vals;
  const float* dinv;
  const float* b;
  VT *r, *z, *p0, *p1, *q;
  VT *rhat, *v, *y, *t;  // BiCGSTAB
  double* x;
  float* xout;
  KScalars* sc;
  double* part;       // [2][4][gridDim.x] block sums
  unsigned* barrier;  // [2] arrivals, generation (zero at launch)
  double rtol;
  int maxiter;
};

// Bounded grid barrier: the last block to arrive bumps the generation the
// others poll; a wait that exceeds its poll limit returns false.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned nblocks, int* s_flag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = bar + 1;
    const unsigned g = *gen;
    int ok = 1;
    __threadfence();
    if (atomicAdd(bar, 1u) == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      for (int i = 0; *gen == g; ++i) {
        if (i >= (1 << 22)) {
          ok = 0;
          break;
        }
        if (i >= 32) __nanosleep(64);
      }
    }
    __threadfence();
    *s_flag = ok;
  }
  __syncthreads();
  const bool ok = *s_flag != 0;
  __syncthreads();
  return ok;
}

// sum of K doubles over the grid, the same totals in every thread of every
// block (block sums added in block order); false if a barrier gave up
template <int K, class Args>
__device__ __forceinline__ bool grid_sum(double (&v)[K], double* sh, const Args& A, int& parity, int* s_flag,
                                         double* s_bcast) {
  const unsigned nb = gridDim.x;
  double* slot = A.part + (size_t)parity * 4 * nb;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const double s = block_sum_d(v[k], sh);
    if (threadIdx.x == 0) __stcg(slot + (size_t)k * nb + blockIdx.x, s);
  }
  if (!grid_barrier(A.barrier, nb, s_flag)) return false;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double t = 0.0;
    for (unsigned i = threadIdx.x; i < nb; i += blockDim.x) t += __ldcg(slot + (size_t)k * nb + i);
    t = block_sum_d(t, sh);
    if (threadIdx.x == 0) s_bcast[k] = t;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = s_bcast[k];
  __syncthreads();
  parity ^= 1;
  return true;
}

template <int NDOF, int G, class T, class Args, class Col, class Epi>
__device__ __forceinline__ void grid_rows(const Args& A, int64_t n0, int64_t n1, Col col, Epi epi) {
  constexpr int U = RowsU<NDOF>::U;
  const int lane = threadIdx.x % G;
  const int64_t group = threadIdx.x / G, ngroups = blockDim.x / G;
  for (int64_t base = n0 + group * U; __any_sync(0xffffffffu, base < n1); base += ngroups * U) {
    T sum;
    int64_t d;
    if (rows_multi<NDOF, G, T>(n1, A.adj_ptr, A.adj, A.vals, A.maxdeg, base, lane, col, sum, d)) epi(d, sum);
  }
}

template <int NDOF, int G, class VT>
__global__ void __launch_bounds__(kGridThreads, 1) k_pcg_grid(const GridArgs<VT> A) {
  __shared__ double sh[32];
  __shared__ double s_bcast[4];
  __shared__ int s_flag;
  int parity = 0;
  const int rank = blockIdx.x, nr = gridDim.x;
  const int64_t n0 = A.N * rank / nr, n1 = A.N * (rank + 1) / nr;
  const int64_t d0 = NDOF * n0, d1 = NDOF * n1;
  const int64_t tid = threadIdx.x, nth = blockDim.x;
  // init: x = 0, r = b, z = D^-1 b, p = 0
  VT rz0 = VT(0), bb0 = VT(0);
  for (int64_t d = d0 + tid; d < d1; d += nth) {
    const VT bi = (VT)A.b[d];
    const VT zi = (VT)A.dinv[d] * bi;
    A.x[d] = 0.0;
    A.r[d] = bi;
    A.z[d] = zi;
    A.p0[d] = VT(0);
    rz0 = vfma(bi, zi, rz0);
    bb0 = vfma(bi, bi, bb0);
  }
  double red[2] = {(double)bb0, (double)rz0};
  int done = 0;
  if (!grid_sum<2>(red, sh, A, parity, &s_flag, s_bcast)) done = 5;
  const double bb = red[0];
  const double tol2 = A.rtol * A.rtol * bb;
  double rho = red[1], rref2 = bb, rnorm2 = bb;
  double alpha = 0.0, beta = 0.0;
  if (!done) done = (bb == 0.0) ? 1 : (!isfinite(bb) ? 3 : 0);
  int iters = 0, breakdowns = 0, replace = 0, cur = 0;
  while (!done) {
    if (!replace) {
      const VT* pold = cur ? A.p1 : A.p0;
      VT* pnew = cur ? A.p0 : A.p1;
      const VT vb = (VT)beta;
      // B: p_new = z + beta p_old (columns on the fly), q = A p_new, p . q
      VT pq = VT(0);
      grid_rows<NDOF, G, VT>(
          A, n0, n1, [&](int64_t k) { return vfma(vb, __ldcg(pold + k), __ldcg(A.z + k)); },
          [&](int64_t d, VT sum) {
            const VT pn = vfma(vb, __ldcg(pold + d), __ldcg(A.z + d));
            __stcg(pnew + d, pn);
            __stcg(A.q + d, sum);
            pq = vfma(pn, sum, pq);
          });
      double dq[1] = {(double)pq};
      if (!grid_sum<1>(dq, sh, A, parity, &s_flag, s_bcast)) {
        done = 5;
        break;
      }
      const double PQ = dq[0];
      if (!(PQ > 0.0) || !isfinite(PQ)) {
        ++breakdowns;
        if (!isfinite(PQ)) done = 3;
        else if (breakdowns > kMaxBreakdowns) done = 4;
        else replace = 2;
        continue;
      }
      alpha = rho / PQ;
      // C: x += alpha p_new, r -= alpha q, z = D^-1 r, r . z, r . r
      const VT va = (VT)alpha;
      VT rz = VT(0), rr = VT(0);
      for (int64_t d = d0 + tid; d < d1; d += nth) {
        const VT pn = __ldcg(pnew + d);
        A.x[d] = fma(alpha, (double)pn, A.x[d]);
        const VT ri = vfma(-va, __ldcg(A.q + d), __ldcg(A.r + d));
        __stcg(A.r + d, ri);
        const VT zi = (VT)A.dinv[d] * ri;
        __stcg(A.z + d, zi);
        rz = vfma(ri, zi, rz);
        rr = vfma(ri, ri, rr);
      }
      double dc[2] = {(double)rz, (double)rr};
      if (!grid_sum<2>(dc, sh, A, parity, &s_flag, s_bcast)) {
        done = 5;
        break;
      }
      const double RZ = dc[0], RR = dc[1];
      beta = RZ / rho;
      rho = RZ;
      rnorm2 = RR;
      ++iters;
      breakdowns = 0;
      cur ^= 1;
      if (!isfinite(RR)) done = 3;
      else if (RR <= tol2 || RR <= kReplaceDrop2 * rref2 || RR > kDiverge2 * bb) replace = 1;
      if (!done && iters >= A.maxiter) replace = replace ? replace : 1;
      if (done || !replace) continue;
    }
    // reliable update: r = b - A x in fp64 (every block's x is visible: the
    // last grid sum ordered it); the direction is kept unless a breakdown
    VT rzf = VT(0);
    double rr = 0.0;
    grid_rows<NDOF, G, double>(A, n0, n1, [&](int64_t k) { return __ldcg(A.x + k); }, [&](int64_t d, double sum) {
      const double ri = (double)A.b[d] - sum;
      const VT rv = (VT)ri;
      __stcg(A.r + d, rv);
      const VT zi = (VT)A.dinv[d] * rv;
      __stcg(A.z + d, zi);
      rzf = vfma(rv, zi, rzf);
      rr = fma(ri, ri, rr);
    });
    double dr[2] = {(double)rzf, rr};
    if (!grid_sum<2>(dr, sh, A, parity, &s_flag, s_bcast)) {
      done = 5;
      break;
    }
    beta = (replace == 2 || !(rho > 0.0) || beta == 0.0) ? 0.0 : dr[0] * beta / rho;
    rho = dr[0];
    rref2 = rnorm2 = dr[1];
    replace = 0;
    if (!isfinite(dr[1])) done = 3;
    else if (dr[1] <= tol2) done = 1;
    else if (dr[1] > kDiverge2 * bb) done = 4;
    else if (iters >= A.maxiter) done = 2;
  }
  for (int64_t d = d0 + tid; d < d1; d += nth) A.xout[d] = (float)A.x[d];
  if (rank == 0 && threadIdx.x == 0) {
    A.sc->iters = iters;
    A.sc->done = done;
    A.sc->rnorm2 = rnorm2;
    A.sc->bnorm2 = bb;
  }
}

// Grid-resident BiCGSTAB: the whole solve in one cooperative launch, as the
// grid CG above and with the cluster solver's iteration (right Jacobi
// preconditioning: y = D^-1 p, z = D^-1 s; fp64 dots and iterate; reliable
// updates from the fp64 iterate, a breakdown restarting the shadow residual).
// Each block owns a contiguous node range; the phases are separated by the
// bounded grid barrier and every reduction is the grid sum in block order, so
// all blocks hold the same scalars.  Vectors another block wrote are read
// through L2 (ld.global.cg).
template <int NDOF, int G, class VT>
__global__ void __launch_bounds__(kGridThreads, 1) k_bicg_grid(const GridArgs<VT> A) {
  __shared__ double sh[32];
  __shared__ double s_bcast[4];
  __shared__ int s_flag;
  int parity = 0;
  const int rank = blockIdx.x, nr = gridDim.x;
  const int64_t n0 = A.N * rank / nr, n1 = A.N * (rank + 1) / nr;
  const int64_t d0 = NDOF * n0, d1 = NDOF * n1;
  const int64_t tid = threadIdx.x, nth = blockDim.x;
  // init: x = 0, r = rhat = b
  double red[1] = {0.0};
  for (int64_t d = d0 + tid; d < d1; d += nth) {
    const float bi = A.b[d];
    A.x[d] = 0.0;
    __stcg(A.r + d, (VT)bi);
    __stcg(A.rhat + d, (VT)bi);
    red[0] += (double)bi * (double)bi;
  }
  int done = 0;
  if (!grid_sum<1>(red, sh, A, parity, &s_flag, s_bcast)) done = 5;
  const double bb = red[0];
  const double tol2 = A.rtol * A.rtol * bb;
  double rho = bb, rref2 = bb, rnorm2 = bb;
  double alpha = 1.0, beta = 0.0, omega = 1.0;
  if (!done) done = (bb == 0.0) ? 1 : (!isfinite(bb) ? 3 : 0);
  int iters = 0, breakdowns = 0, replace = 0;
  bool restart = true;
  while (!done) {
    if (!replace) {
      // A: p = r + beta (p - omega v) (p = r on restart), y = D^-1 p
      const VT vb = (VT)beta, vo = (VT)omega;
      for (int64_t d = d0 + tid; d < d1; d += nth) {
        const VT rd = __ldcg(A.r + d);
        const VT pn = restart ? rd : vfma(vb, vfma(-vo, __ldcg(A.v + d), __ldcg(A.p0 + d)), rd);
        __stcg(A.p0 + d, pn);
        __stcg(A.y + d, (VT)A.dinv[d] * pn);
      }
      if (!grid_barrier(A.barrier, nr, &s_flag)) {
        done = 5;
        break;
      }
      // B: v = A y, rhat . v
      double dv[1] = {0.0};
      grid_rows<NDOF, G, VT>(A, n0, n1, [&](int64_t k) { return __ldcg(A.y + k); }, [&](int64_t d, VT sum) {
        __stcg(A.v + d, sum);
        dv[0] += (double)__ldcg(A.rhat + d) * (double)sum;
      });
      if (!grid_sum<1>(dv, sh, A, parity, &s_flag, s_bcast)) {
        done = 5;
        break;
      }
      const double RV = dv[0];
      restart = false;
      if (RV == 0.0 || !isfinite(RV)) {
        ++breakdowns;
        if (!isfinite(RV)) done = 3;
        else if (breakdowns > kMaxBreakdowns) done = 4;
        else replace = 2;
        continue;
      }
      alpha = rho / RV;
      // C: s = r - alpha v (kept in q), z = D^-1 s
      const VT va = (VT)alpha;
      for (int64_t d = d0 + tid; d < d1; d += nth) {
        const VT sv = vfma(-va, __ldcg(A.v + d), __ldcg(A.r + d));
        __stcg(A.q + d, sv);
        __stcg(A.z + d, (VT)A.dinv[d] * sv);
      }
      if (!grid_barrier(A.barrier, nr, &s_flag)) {
        done = 5;
        break;
      }
      // D: t = A z, t . s, t . t
      double dt[2] = {0.0, 0.0};
      grid_rows<NDOF, G, VT>(A, n0, n1, [&](int64_t k) { return __ldcg(A.z + k); }, [&](int64_t d, VT sum) {
        __stcg(A.t + d, sum);
        dt[0] += (double)sum * (double)__ldcg(A.q + d);
        dt[1] += (double)sum * (double)sum;
      });
      if (!grid_sum<2>(dt, sh, A, parity, &s_flag, s_bcast)) {
        done = 5;
        break;
      }
      omega = (dt[1] > 0.0 && isfinite(dt[1])) ? dt[0] / dt[1] : 0.0;
      // E: x += alpha y + omega z, r = s - omega t, rhat . r, r . r
      const VT vom = (VT)omega;
      double de[2] = {0.0, 0.0};
      for (int64_t d = d0 + tid; d < d1; d += nth) {
        A.x[d] = fma(omega, (double)__ldcg(A.z + d), fma(alpha, (double)__ldcg(A.y + d), A.x[d]));
        const VT ri = vfma(-vom, __ldcg(A.t + d), __ldcg(A.q + d));
        __stcg(A.r + d, ri);
        de[0] += (double)__ldcg(A.rhat + d) * (double)ri;
        de[1] += (double)ri * (double)ri;
      }
      if (!grid_sum<2>(de, sh, A, parity, &s_flag, s_bcast)) {
        done = 5;
        break;
      }
      const double RH = de[0], RR = de[1];
      beta = (omega != 0.0 && rho != 0.0) ? (RH / rho) * (alpha / omega) : 0.0;
      rho = RH;
      rnorm2 = RR;
      ++iters;
      breakdowns = 0;
      if (!isfinite(RR)) done = 3;
      else if (RH == 0.0 || omega == 0.0) replace = 2;
      else if (RR <= tol2 || RR <= kReplaceDrop2 * rref2 || RR > kDiverge2 * bb) replace = 1;
      if (!done && iters >= A.maxiter) replace = replace ? replace : 1;
      if (done || !replace) continue;
    }
    // reliable update: r = b - A x in fp64 (every block's x is visible: the
    // last grid sum ordered it); a breakdown (replace == 2) also restarts the
    // shadow residual
    const bool fresh = replace == 2;
    double dr[2] = {0.0, 0.0};
    grid_rows<NDOF, G, double>(A, n0, n1, [&](int64_t k) { return __ldcg(A.x + k); }, [&](int64_t d, double sum) {
      const double ri = (double)A.b[d] - sum;
      const VT rv = (VT)ri;
      __stcg(A.r + d, rv);
      if (fresh) {
        __stcg(A.rhat + d, rv);
        dr[0] += (double)rv * (double)rv;
      } else {
        dr[0] += (double)__ldcg(A.rhat + d) * (double)rv;
      }
      dr[1] += ri * ri;
    });
    if (!grid_sum<2>(dr, sh, A, parity, &s_flag, s_bcast)) {
      done = 5;
      break;
    }
    rho = dr[0];
    rref2 = rnorm2 = dr[1];
    if (fresh) restart = true;
    replace = 0;
    if (!isfinite(dr[1])) done = 3;
    else if (dr[1] <= tol2) done = 1;
    else if (dr[1] > kDiverge2 * bb) done = 4;
    else if (iters >= A.maxiter) done = 2;
  }
  for (int64_t d = d0 + tid; d < d1; d += nth) A.xout[d] = (float)A.x[d];
  if (rank == 0 && threadIdx.x == 0) {
    A.sc->iters = iters;
    A.sc->done = done;
    A.sc->rnorm2 = rnorm2;
    A.sc->bnorm2 = bb;
  }
}

// one cooperative launch of the grid solver (every block resident); returns
// false if the launch was refused (the caller then uses the multi-kernel path)
template <int NDOF, int G, class VT, bool BICG = false>
static bool launch_grid_pcg(const GridArgs<VT>& A, cudaStream_t s) {
  auto kernel = BICG ? k_bicg_grid<NDOF, G, VT> : k_pcg_grid<NDOF, G, VT>;
  static std::atomic<int> occ[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
  int per_sm = occ[dev].load();
  if (per_sm == 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kGridThreads, 0) != cudaSuccess ||
        per_sm < 1) {
      cudaGetLastError();
      return false;
    }
    occ[dev].store(per_sm);
  }
  const int64_t want = (A.N + 63) / 64;  // at least 64 nodes per block
  int64_t blocks = (int64_t)per_sm * num_sms();
  if (blocks > want) blocks = want;
  if (blocks < 1 || blocks > 8192) return false;  // part holds [2][4][blocks] doubles
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3(kGridThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, kernel, A) == cudaSuccess) return true;
  cudaGetLastError();
  return false;
}

// capture_sc != NULL: s is being captured into a graph (the device-resident
// Newton solve, the cached graphs of krylov_async); the solve is enqueued as
// init + one WHILE node over [K iterations, true residual, loop control] (or
// one cluster launch for small fp32 systems) + the fp32 copy of x, with no
// host synchronisation, and *capture_sc receives the solver's device scalars.
// capture_sc == NULL: the host-driven loop (one flag read per check_every
// iterations), used while kernel tracing is on.
template <class VT>
static int krylov_solve(const folgb_plan* p, int solver, const float* vals, const float* dinv, const float* rhs,
                        float* x, double rtol, int maxiter, int check_every, int32_t* iterations,
                        double* rel_residual, void* workspace, size_t workspace_bytes, cudaStream_t s,
                        KScalars** capture_sc = nullptr) {
  if (!p || !vals || !dinv || !rhs || !x || maxiter <= 0 || !(rtol >= 0.0)) return FOLGB_ERR_INVALID_ARGUMENT;
  if (!p->has_csr) return FOLGB_ERR_NO_PATTERN;
  KWork<VT> w;
  size_t need = layout_krylov<VT>(p, workspace, workspace_bytes, &w);
  if (!workspace || workspace_bytes < need) return FOLGB_ERR_WORKSPACE;
  if (check_every <= 0) check_every = 32;
  const int64_t n = (int64_t)p->ndof * p->N;
  int vb = (int)((n + 255) / 256);
  if (vb > kVecBlocks) vb = kVecBlocks;
  // the PCG update: 2 blocks per SM, 4 entries per thread per trip (few
  // blocks keep the last-block-done counter, one atomic per block, cheap)
  int ub = (int)((n + 1023) / 1024);
  if (ub > 2 * num_sms()) ub = 2 * num_sms();
  FOLGB_CUDA_TRY(cudaMemsetAsync(w.counters, 0, 8 * sizeof(unsigned), s));
  if (solver == SOLVER_CG)
    k_pcg_init<VT><<<vb, 256, 0, s>>>(n, rhs, dinv, w.x, w.r, w.z, w.p0, w.part, w.counters, w.sc, rtol, maxiter);
  else
    k_bicg_init<VT><<<vb, 256, 0, s>>>(n, rhs, w.x, w.r, w.rhat, w.part, w.counters, w.sc, rtol, maxiter);
  FOLGB_LAUNCH_CHECK();
  KScalars host{};
  int rc = with_ndof(p->ndof, [&](auto nd) -> int {
    constexpr int NDOF = decltype(nd)::value;
    return with_group<NDOF>(p->maxdeg, [&](auto gw) -> int {
      constexpr int G = decltype(gw)::value;
      const int sb = spmv_blocks<NDOF>(p, G);
      // one chunk of iterations on stream cs (the kernels pick the current
      // direction buffers from the device scalars)
      auto chunk = [&](int count, cudaStream_t cs) {
        for (int k = 0; k < count; ++k) {
          if (solver == SOLVER_CG) {
            trace_begin(KID_PCG_SPMV, cs);
            k_pcg_spmv<NDOF, G, VT><<<sb, 256, 0, cs>>>(p->N, p->d_adj_ptr, p->d_adj, p->maxdeg, vals, w.z, w.p0,
                                                     w.p1, w.q, w.part, w.counters, w.sc);
            trace_end(KID_PCG_SPMV, cs);
            trace_begin(KID_PCG_UPDATE, cs);
            k_pcg_update<VT><<<ub, 256, 0, cs>>>(n, dinv, w.x, w.r, w.z, w.p0, w.p1, w.q, w.part, w.counters, w.sc);
            trace_end(KID_PCG_UPDATE, cs);
          } else {
            trace_begin(KID_PCG_SPMV, cs);
            k_bicg_p_spmv<NDOF, G, VT><<<sb, 256, 0, cs>>>(p->N, p->d_adj_ptr, p->d_adj, p->maxdeg, vals, dinv, w.r,
                                                        w.rhat, w.p0, w.p1, w.v0, w.v1, w.y, w.part, w.counters,
                                                        w.sc);
            k_bicg_s_spmv<NDOF, G, VT><<<sb, 256, 0, cs>>>(p->N, p->d_adj_ptr, p->d_adj, p->maxdeg, vals, dinv, w.r,
                                                        w.v0, w.v1, w.z, w.t, w.part, w.counters, w.sc);
            trace_end(KID_PCG_SPMV, cs);
            trace_begin(KID_PCG_UPDATE, cs);
            k_bicg_update<VT><<<vb, 256, 0, cs>>>(n, w.x, w.r, w.rhat, w.v0, w.v1, w.y, w.z, w.t, w.part, w.counters,
                                                  w.sc);
            trace_end(KID_PCG_UPDATE, cs);
          }
        }
      };
      auto true_residual = [&](cudaStream_t cs) {
        if (solver == SOLVER_CG)
          k_true_residual<NDOF, G, false, VT><<<sb, 256, 0, cs>>>(p->N, p->d_adj_ptr, p->d_adj, p->maxdeg, vals,
                                                                 rhs, dinv, w.x, w.r, w.z, w.rhat, w.part,
                                                                 w.counters, w.sc);
        else
          k_true_residual<NDOF, G, true, VT><<<sb, 256, 0, cs>>>(p->N, p->d_adj_ptr, p->d_adj, p->maxdeg, vals,
                                                                rhs, dinv, w.x, w.r, w.z, w.rhat, w.part,
                                                                w.counters, w.sc);
      };
      const int K = (check_every + 1) & ~1;
      const int max_rounds = 4 * (maxiter / K + 8);
      auto cluster_args = [&]() {
        ClusterArgs<VT> ca;
        ca.N = p->N;
        ca.adj_ptr = p->d_adj_ptr;
        ca.adj = p->d_adj;
        ca.maxdeg = p->maxdeg;
        ca.vals = vals;
        ca.dinv = dinv;
        ca.b = rhs;
        ca.r = w.r;
        ca.z = w.z;
        ca.p = w.p0;
        ca.q = w.q;
        ca.rhat = w.rhat;
        ca.v = w.v0;
        ca.y = w.y;
        ca.t = w.t;
        ca.x = w.x;
        ca.xout = x;
        ca.sc = w.sc;
        ca.rtol = rtol;
        ca.maxiter = maxiter;
        return ca;
      };
      if (capture_sc) {
        // small fp32 systems: the whole solve is one cluster launch here too
        if (n <= kClusterMaxDofs && sizeof(VT) == sizeof(float) &&
            launch_cluster_solver<NDOF, G, VT>(solver, cluster_args(), s)) {
          *capture_sc = w.sc;
          return (int)FOLGB_OK;
        }
        // large fp32 CG systems: one cooperative launch of the grid solver
        if (solver == SOLVER_CG && n > kClusterMaxDofs && sizeof(VT) == sizeof(float) &&
            krylov_engine() == FOLGB_KRYLOV_ENGINE_GRID) {
          GridArgs<VT> ga;
          ga.N = p->N;
          ga.adj_ptr = p->d_adj_ptr;
          ga.adj = p->d_adj;
          ga.maxdeg = p->maxdeg;
          ga.vals = vals;
          ga.dinv = dinv;
          ga.b = rhs;
          ga.r = w.r;
          ga.z = w.z;
          ga.p0 = w.p0;
          ga.p1 = w.p1;
          ga.q = w.q;
          ga.x = w.x;
          ga.xout = x;
          ga.sc = w.sc;
          ga.part = w.part;
          ga.barrier = w.counters + 6;
          ga.rtol = rtol;
          ga.maxiter = maxiter;
          if (launch_grid_pcg<NDOF, G, VT>(ga, s)) {
            *capture_sc = w.sc;
            return (int)FOLGB_OK;
          }
        }
        // BiCGSTAB with fp64 vectors (the neo-Hookean Newton solves) above
        // 32,768 dofs: one cooperative launch of the grid solver (24^3 tet
        // split, 46,875 dofs: 68 us per iteration against 74 in the kernel
        // loop; 16^3, 14,739 dofs: 53 against 37, the grid barriers dominate
        // there).  fp32 vectors stay on the kernel loop: their iteration count
        // swings with the reduction order (24^3 elasticity: 644 iterations in
        // the grid solver against 417), with fp64 vectors it does not.
        if (solver == SOLVER_BICGSTAB && sizeof(VT) == sizeof(double) && n > 2 * kClusterMaxDofs &&
            krylov_engine() == FOLGB_KRYLOV_ENGINE_GRID) {
          GridArgs<VT> ga;
          ga.N = p->N;
          ga.adj_ptr = p->d_adj_ptr;
          ga.adj = p->d_adj;
          ga.maxdeg = p->maxdeg;
          ga.vals = vals;
          ga.dinv = dinv;
          ga.b = rhs;
          ga.r = w.r;
          ga.z = w.z;
          ga.p0 = w.p0;
          ga.p1 = w.p1;
          ga.q = w.q;
          ga.rhat = w.rhat;
          ga.v = w.v0;
          ga.y = w.y;
          ga.t = w.t;
          ga.x = w.x;
          ga.xout = x;
          ga.sc = w.sc;
          ga.part = w.part;
          ga.barrier = w.counters + 6;
          ga.rtol = rtol;
          ga.maxiter = maxiter;
          if (launch_grid_pcg<NDOF, G, VT, true>(ga, s)) {
            *capture_sc = w.sc;
            return (int)FOLGB_OK;
          }
        }
        cudaStreamCaptureStatus cst = cudaStreamCaptureStatusNone;
        cudaGraph_t graph = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        FOLGB_CUDA_TRY(cudaStreamGetCaptureInfo(s, &cst, nullptr, &graph, &deps, nullptr, &ndeps));
        if (cst != cudaStreamCaptureStatusActive) return (int)FOLGB_ERR_INVALID_ARGUMENT;
        cudaGraphConditionalHandle loop{};
        FOLGB_CUDA_TRY(cudaGraphConditionalHandleCreate(&loop, graph, 1u, cudaGraphCondAssignDefault));
        // the default value is assigned only when the top-level graph is
        // launched: re-arm the loop each time the enclosing body runs
        k_arm_conditional<<<1, 32, 0, s>>>(loop);
        FOLGB_LAUNCH_CHECK();
        FOLGB_CUDA_TRY(cudaStreamGetCaptureInfo(s, &cst, nullptr, &graph, &deps, nullptr, &ndeps));
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = loop;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        FOLGB_CUDA_TRY(cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &np));
        FOLGB_CUDA_TRY(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
        cudaStream_t cs = nullptr;
        FOLGB_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        int crc = FOLGB_OK;
        if (cudaStreamBeginCaptureToGraph(cs, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeRelaxed) != cudaSuccess) {
          crc = FOLGB_ERR_CUDA;
        } else {
          chunk(K, cs);
          true_residual(cs);
          k_krylov_continue<<<1, 32, 0, cs>>>(w.sc, loop, maxiter, max_rounds);
          const bool launched_ok = cudaGetLastError() == cudaSuccess;
          cudaGraph_t body_out = nullptr;
          if (cudaStreamEndCapture(cs, &body_out) != cudaSuccess || !launched_ok) crc = FOLGB_ERR_CUDA;
        }
        cudaStreamDestroy(cs);
        if (crc) return crc;
        k_to_float<<<vb, 256, 0, s>>>(n, w.x, x);
        FOLGB_LAUNCH_CHECK();
        *capture_sc = w.sc;
        return (int)FOLGB_OK;
      }
      // host-driven loop (the synchronous entry points while kernel tracing
      // is on: every launch gets its events); otherwise the solve is a cached
      // graph (krylov_async)
      int guard = 0;
      while (true) {
        chunk(check_every, s);
        FOLGB_LAUNCH_CHECK();
        FOLGB_CUDA_TRY(cudaMemcpyAsync(&host, w.sc, sizeof(KScalars), cudaMemcpyDeviceToHost, s));
        FOLGB_CUDA_TRY(cudaStreamSynchronize(s));
        if (host.done) break;
        if (host.replace) {
          true_residual(s);
          FOLGB_LAUNCH_CHECK();
          FOLGB_CUDA_TRY(cudaMemcpyAsync(&host, w.sc, sizeof(KScalars), cudaMemcpyDeviceToHost, s));
          FOLGB_CUDA_TRY(cudaStreamSynchronize(s));
          if (host.done) break;
          if (host.iters >= maxiter) {
            host.done = 2;
            break;
          }
        }
        // hard cap on host rounds (each round runs >= 1 iteration or a replacement)
        if (++guard > 4 * (maxiter / check_every + 8)) {
          host.done = 2;
          break;
        }
      }
      k_to_float<<<vb, 256, 0, s>>>(n, w.x, x);
      FOLGB_LAUNCH_CHECK();
      return (int)FOLGB_OK;
    });
  });
  if (rc || capture_sc) return rc;
  if (iterations) *iterations = host.iters;
  if (rel_residual) *rel_residual = host.bnorm2 > 0 ? std::sqrt(host.rnorm2 / host.bnorm2) : 0.0;
  if (host.done == 3) return FOLGB_ERR_NAN;
  if (host.done != 1) return FOLGB_ERR_NOT_CONVERGED;
  return FOLGB_OK;
}

__global__ void k_krylov_report(const KScalars* sc, int32_t* iterations, double* rel_residual, int32_t* status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (iterations) *iterations = sc->iters;
  if (rel_residual) *rel_residual = sc->bnorm2 > 0.0 ? sqrt(sc->rnorm2 / sc->bnorm2) : 0.0;
  if (status)
    *status = sc->done == 3 ? FOLGB_ERR_NAN
                            : (sc->done == 1 ? FOLGB_OK : (sc->done == 5 ? FOLGB_ERR_TIMEOUT : FOLGB_ERR_NOT_CONVERGED));
}

// Instantiated solve graphs of one plan, keyed by everything the graph bakes
// in (buffers, method, precision, tolerance, iteration limits, device); the
// oldest entry is dropped past kKrylovGraphs.
struct KrylovGraphKey {
  const void* ptrs[9];
  int solver, vbits, maxiter, check_every, device, engine;
  double rtol;
  bool operator==(const KrylovGraphKey& o) const {
    for (int i = 0; i < 9; ++i)
      if (ptrs[i] != o.ptrs[i]) return false;
    return solver == o.solver && vbits == o.vbits && maxiter == o.maxiter && check_every == o.check_every &&
           device == o.device && engine == o.engine && rtol == o.rtol;
  }
};
struct KrylovGraphs {
  std::mutex mu;
  std::vector<std::pair<KrylovGraphKey, cudaGraphExec_t>> entries;
};
constexpr size_t kKrylovGraphs = 8;

void free_krylov_graphs(folgb_plan* p) {
  auto* c = static_cast<KrylovGraphs*>(p->krylov_graphs);
  if (!c) return;
  for (auto& e : c->entries) cudaGraphExecDestroy(e.second);
  delete c;
  p->krylov_graphs = nullptr;
}

static std::mutex g_krylov_cache_create;

// Enqueues the whole solve on s with no host synchronisation: init, the WHILE
// loop, the fp32 copy of x and the report into the caller's device buffers.
// A stream under capture gets the nodes added to its graph; otherwise the
// solve runs as a cached instantiated graph (built on the first call with
// these arguments: capture on a private stream + instantiate).
template <class VT>
static int krylov_async(const folgb_plan* p, int solver, const float* vals, const float* dinv, const float* rhs,
                        float* x, double rtol, int maxiter, int check_every, int32_t* d_iterations,
                        double* d_rel_residual, int32_t* d_status, void* workspace, size_t workspace_bytes,
                        cudaStream_t s) {
  if (!p || !vals || !dinv || !rhs || !x || maxiter <= 0 || !(rtol >= 0.0)) return FOLGB_ERR_INVALID_ARGUMENT;
  if (!p->has_csr) return FOLGB_ERR_NO_PATTERN;
  if (!workspace || workspace_bytes < layout_krylov<VT>(p, nullptr, 0, nullptr)) return FOLGB_ERR_WORKSPACE;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  FOLGB_CUDA_TRY(cudaStreamIsCapturing(s, &cap));
  if (cap == cudaStreamCaptureStatusActive) {
    KScalars* sc = nullptr;
    int rc = krylov_solve<VT>(p, solver, vals, dinv, rhs, x, rtol, maxiter, check_every, nullptr, nullptr, workspace,
                              workspace_bytes, s, &sc);
    if (rc) return rc;
    k_krylov_report<<<1, 32, 0, s>>>(sc, d_iterations, d_rel_residual, d_status);
    FOLGB_LAUNCH_CHECK();
    return FOLGB_OK;
  }
  KrylovGraphKey key{};
  const void* ptrs[9] = {vals, dinv, rhs, x, workspace, d_iterations, d_rel_residual, d_status,
                         reinterpret_cast<const void*>(workspace_bytes)};
  for (int i = 0; i < 9; ++i) key.ptrs[i] = ptrs[i];
  key.solver = solver;
  key.vbits = (int)(8 * sizeof(VT));
  key.maxiter = maxiter;
  key.check_every = check_every;
  key.rtol = rtol;
  key.engine = krylov_engine();
  FOLGB_CUDA_TRY(cudaGetDevice(&key.device));
  folgb_plan* mp = const_cast<folgb_plan*>(p);  // the cache is the plan's only mutable state
  {
    std::lock_guard<std::mutex> g(g_krylov_cache_create);
    if (!mp->krylov_graphs) mp->krylov_graphs = new KrylovGraphs();
  }
  auto* cache = static_cast<KrylovGraphs*>(mp->krylov_graphs);
  std::lock_guard<std::mutex> lock(cache->mu);
  cudaGraphExec_t exec = nullptr;
  for (auto& e : cache->entries)
    if (e.first == key) exec = e.second;
  if (!exec) {
    cudaStream_t cs = nullptr;
    FOLGB_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    int rc = FOLGB_OK;
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      rc = FOLGB_ERR_CUDA;
    } else {
      KScalars* sc = nullptr;
      rc = krylov_solve<VT>(p, solver, vals, dinv, rhs, x, rtol, maxiter, check_every, nullptr, nullptr, workspace,
                            workspace_bytes, cs, &sc);
      if (rc == FOLGB_OK) {
        k_krylov_report<<<1, 32, 0, cs>>>(sc, d_iterations, d_rel_residual, d_status);
        if (cudaGetLastError() != cudaSuccess) rc = FOLGB_ERR_CUDA;
      }
      if (cudaStreamEndCapture(cs, &graph) != cudaSuccess && rc == FOLGB_OK) rc = FOLGB_ERR_CUDA;
    }
    if (rc == FOLGB_OK && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) rc = FOLGB_ERR_CUDA;
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (rc) {
      cudaGetLastError();
      return rc;
    }
    if (cache->entries.size() >= kKrylovGraphs) {
      cudaGraphExecDestroy(cache->entries.front().second);
      cache->entries.erase(cache->entries.begin());
    }
    cache->entries.emplace_back(key, exec);
  }
  FOLGB_CUDA_TRY(cudaGraphLaunch(exec, s));
  return FOLGB_OK;
}

// The synchronous entry points: the stream-ordered solve, then one read of
// its report (or, while kernel tracing is on, the host-driven loop).
template <class VT>
static int krylov_sync(const folgb_plan* p, int solver, const float* vals, const float* dinv, const float* rhs,
                       float* x, double rtol, int maxiter, int check_every, int32_t* iterations,
                       double* rel_residual, void* workspace, size_t workspace_bytes, cudaStream_t s) {
  if (trace_active())
    return krylov_solve<VT>(p, solver, vals, dinv, rhs, x, rtol, maxiter, check_every, iterations, rel_residual,
                            workspace, workspace_bytes, s);
  KWork<VT> w;
  if (!p || !workspace || workspace_bytes < layout_krylov<VT>(p, workspace, workspace_bytes, &w))
    return p ? FOLGB_ERR_WORKSPACE : FOLGB_ERR_INVALID_ARGUMENT;
  int rc = krylov_async<VT>(p, solver, vals, dinv, rhs, x, rtol, maxiter, check_every, &w.report->iterations,
                            &w.report->rel_residual, &w.report->status, workspace, workspace_bytes, s);
  if (rc) return rc;
  KReport host{};
  FOLGB_CUDA_TRY(cudaMemcpyAsync(&host, w.report, sizeof(KReport), cudaMemcpyDeviceToHost, s));
  FOLGB_CUDA_TRY(cudaStreamSynchronize(s));
  if (iterations) *iterations = host.iterations;
  if (rel_residual) *rel_residual = host.rel_residual;
  return host.status;
}

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
      k_spmv<NDOF, G><<<spmv_blocks<NDOF>(p, G), 256, 0, s>>>(p->N, p->d_adj_ptr, p->d_adj, p->maxdeg, vals, x, y);
      FOLGB_LAUNCH_CHECK();
      return (int)FOLGB_OK;
    });
  });
}

extern "C" int folgb_pcg(const folgb_plan* p, const float* vals, const float* dinv, const float* rhs, float* x,
                         double rtol, int32_t maxiter, int32_t check_every, int32_t* iterations, double* rel_residual,
                         void* workspace, size_t workspace_bytes, void* stream) {
  return krylov_sync<float>(p, SOLVER_CG, vals, dinv, rhs, x, rtol, maxiter, check_every, iterations, rel_residual,
                            workspace, workspace_bytes, (cudaStream_t)stream);
}

extern "C" int folgb_bicgstab(const folgb_plan* p, const float* vals, const float* dinv, const float* rhs, float* x,
                              double rtol, int32_t maxiter, int32_t check_every, int32_t* iterations,
                              double* rel_residual, void* workspace, size_t workspace_bytes, void* stream) {
  return krylov_sync<float>(p, SOLVER_BICGSTAB, vals, dinv, rhs, x, rtol, maxiter, check_every, iterations,
                            rel_residual, workspace, workspace_bytes, (cudaStream_t)stream);
}

extern "C" int folgb_krylov(const folgb_plan* p, int32_t method, int32_t vector_bits, const float* vals,
                            const float* dinv, const float* rhs, float* x, double rtol, int32_t maxiter,
                            int32_t check_every, int32_t* iterations, double* rel_residual, void* workspace,
                            size_t workspace_bytes, void* stream) {
  if (method != FOLGB_KRYLOV_CG && method != FOLGB_KRYLOV_BICGSTAB) return FOLGB_ERR_INVALID_ARGUMENT;
  const int solver = method == FOLGB_KRYLOV_CG ? SOLVER_CG : SOLVER_BICGSTAB;
  if (vector_bits == 32)
    return krylov_sync<float>(p, solver, vals, dinv, rhs, x, rtol, maxiter, check_every, iterations, rel_residual,
                              workspace, workspace_bytes, (cudaStream_t)stream);
  if (vector_bits == 64)
    return krylov_sync<double>(p, solver, vals, dinv, rhs, x, rtol, maxiter, check_every, iterations, rel_residual,
                               workspace, workspace_bytes, (cudaStream_t)stream);
  return FOLGB_ERR_INVALID_ARGUMENT;
}

extern "C" int folgb_krylov_set_engine(int32_t engine) {
  if (engine != FOLGB_KRYLOV_ENGINE_GRID && engine != FOLGB_KRYLOV_ENGINE_KERNELS) return FOLGB_ERR_INVALID_ARGUMENT;
  g_krylov_engine.store(engine);
  return FOLGB_OK;
}

extern "C" int folgb_krylov_async(const folgb_plan* p, int32_t method, int32_t vector_bits, const float* vals,
                                  const float* dinv, const float* rhs, float* x, double rtol, int32_t maxiter,
                                  int32_t check_every, int32_t* d_iterations, double* d_rel_residual,
                                  int32_t* d_status, void* workspace, size_t workspace_bytes, void* stream) {
  if (method != FOLGB_KRYLOV_CG && method != FOLGB_KRYLOV_BICGSTAB) return FOLGB_ERR_INVALID_ARGUMENT;
  const int solver = method == FOLGB_KRYLOV_CG ? SOLVER_CG : SOLVER_BICGSTAB;
  if (check_every <= 0) check_every = 32;
  if (vector_bits == 32)
    return krylov_async<float>(p, solver, vals, dinv, rhs, x, rtol, maxiter, check_every, d_iterations,
                               d_rel_residual, d_status, workspace, workspace_bytes, (cudaStream_t)stream);
  if (vector_bits == 64)
    return krylov_async<double>(p, solver, vals, dinv, rhs, x, rtol, maxiter, check_every, d_iterations,
                                d_rel_residual, d_status, workspace, workspace_bytes, (cudaStream_t)stream);
  return FOLGB_ERR_INVALID_ARGUMENT;
}

extern "C" int folgb_adam_step(float* params, const float* grads, float* m, float* v, int64_t n, int32_t* step,
                               float lr, float beta1, float beta2, float eps, void* stream) {
  if (!params || !grads || !m || !v || !step || n < 0) return FOLGB_ERR_INVALID_ARGUMENT;
  if (n == 0) return FOLGB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int blocks = (int)((n / 4 + 255) / 256);
  if (blocks < 1) blocks = 1;
  int cap = num_sms() * 8;
  if (blocks > cap) blocks = cap;
  k_adam<<<blocks, 256, 0, s>>>(params, grads, m, v, n, step, lr, beta1, beta2, eps);
  k_step_inc<<<1, 1, 0, s>>>(step);
  FOLGB_LAUNCH_CHECK();
  return FOLGB_OK;
}

// ---------------------------------------------------------------------------
// Device-resident Newton-Raphson with load stepping
// (fol/solvers/fe_nonlinear_residual_based_solver.py:76-170).  The whole solve
// is one CUDA graph: a WHILE node whose body is one Newton iteration
// [load-scaled Dirichlet values at the start of a load step, residual and
// CSR tangent assembly, |r| and rhs = -r, the Krylov solve (a nested WHILE
// node), |du|, the convergence test, (optionally) a backtracking line search
// on the element energy (a nested WHILE node), u += t du], launched once; the
// host reads the Newton state when the graph has finished.  Convergence as
// the reference: |r| < abs_tol or |du| < rel_tol or the iteration cap, the
// converged iteration's update not applied; a non-finite |r| stops the solve.
// ---------------------------------------------------------------------------
namespace folgb {

struct NState {
  double rn2, dn2, abs2, rel2;
  long long krylov_total;
  int step, it, steps, maxit, done, status, newton_total, apply, krylov_fail;
  // line search: slope r . du (r is -rhs), step length t, halvings
  double slope, t;
  int ls_it, ls_max, ls_halvings;
};

constexpr int kNewtonBlocks = 1024;

__global__ void k_newton_bc(int64_t N, int ndof, const unsigned char* __restrict__ dmask,
                            const float* __restrict__ dval, float* __restrict__ u, const NState* st) {
  if (st->it != 0 || st->done) return;  // only at the start of a load step
  const double frac = (double)(st->step + 1) / (double)st->steps;
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const unsigned m = dmask[n];
    for (int c = 0; c < ndof; ++c)
      if ((m >> c) & 1u) u[(int64_t)ndof * n + c] = (float)(frac * (double)dval[(int64_t)ndof * n + c]);
  }
}

// rhs = -r (when neg) and the fp64 squared norm of v into *out, fixed order
__global__ void k_newton_norm(int64_t n, const float* __restrict__ v, float* __restrict__ neg, double* part,
                              unsigned* counter, double* out) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float x = v[i];
    if (neg) neg[i] = -x;
    acc += (double)x * (double)x;
  }
  const double s = block_sum_d(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  if (!last_block(counter)) return;
  const double tot = sum_partials(part, gridDim.x, sh);
  if (threadIdx.x == 0) {
    *out = tot;
    *counter = 0u;
  }
}

// hist[k] = (load step, iteration, |r|, |du|) of Newton iteration k
__global__ void k_newton_control(NState* st, const KScalars* sc, double* hist, int hist_cap) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int k = st->newton_total;
  if (k < hist_cap) {
    hist[4 * k] = st->step + 1;
    hist[4 * k + 1] = st->it + 1;
    hist[4 * k + 2] = sqrt(st->rn2);
    hist[4 * k + 3] = sqrt(st->dn2);
  }
  st->newton_total = k + 1;
  st->krylov_total += sc->iters;
  if (sc->done == 3 || sc->done == 4) st->krylov_fail += 1;
  st->it += 1;
  st->apply = 0;
  if (!isfinite(st->rn2)) {
    st->status = FOLGB_ERR_NAN;
    st->done = 1;
  } else if (st->rn2 < st->abs2 || st->dn2 < st->rel2 || st->it >= st->maxit) {
    st->step += 1;
    st->it = 0;
    if (st->step >= st->steps) st->done = 1;
  } else {
    st->apply = 1;
  }
  // every body execution is one Newton iteration: at most steps * maxit
  if (st->newton_total >= st->steps * st->maxit) st->done = 1;
}

// Last kernel of the Newton body: continue unless the solve has ended (in
// this iteration's control or its line search).
__global__ void k_newton_loop(const NState* st, cudaGraphConditionalHandle loop) {
  if (threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(loop, st->done ? 0u : 1u);
}

__global__ void k_newton_update(int64_t n, float* __restrict__ u, const float* __restrict__ du, const NState* st) {
  if (!st->apply) return;
  const float t = (float)st->t;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    u[i] = t == 1.f ? u[i] + du[i] : fmaf(t, du[i], u[i]);
}

// fp64 dot product a . b into *out, fixed order (the line search's slope)
__global__ void k_newton_dot(int64_t n, const float* __restrict__ a, const float* __restrict__ b, double* part,
                             unsigned* counter, double* out) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc += (double)a[i] * (double)b[i];
  const double s = block_sum_d(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  if (!last_block(counter)) return;
  const double tot = sum_partials(part, gridDim.x, sh);
  if (threadIdx.x == 0) {
    *out = tot;
    *counter = 0u;
  }
}

// Line search (backtracking on the element energy).  Arm: full step, and the
// loop runs only for an iteration whose update is applied and whose
// predicted decrease -(r . du) = slope (rhs = -r, so slope = -(rhs . du))
// is above the energy's fp32 resolution.
__global__ void k_ls_arm(NState* st, const float* e0, cudaGraphConditionalHandle h) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  st->t = 1.0;
  st->ls_it = 0;
  const double pred = st->slope;  // rhs . du = -(r . du): the predicted decrease
  // a tiny predicted decrease (below the energy's fp32 resolution) takes the
  // whole step; a direction that is not a descent one is searched as well
  const bool tiny = pred >= 0.0 && pred <= 1e-6 * fabs((double)*e0);
  const bool run = st->apply && !st->done && !tiny;
  cudaGraphSetConditional(h, run ? 1u : 0u);
}

// A Newton step that is not a descent direction (indefinite tangent: slope
// = rhs . du <= 0), that the Krylov solve left non-finite, or whose Krylov
// solve did not converge (an unconverged iterate on an indefinite system can
// be a descent direction of useless length) is replaced by the
// Jacobi-preconditioned steepest descent step du = D^-1 rhs = -D^-1 r.
__global__ void k_ls_direction(int64_t n, const float* __restrict__ rhs, const float* __restrict__ dinv,
                               float* __restrict__ du, const NState* st, const KScalars* sc) {
  const double sl = st->slope;
  const bool failed = sc && (sc->done == 3 || sc->done == 4);
  if (isfinite(sl) && sl > 0.0 && !failed) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    du[i] = dinv[i] * rhs[i];
}

__global__ void k_ls_trial(int64_t n, const float* __restrict__ u, const float* __restrict__ du, float* __restrict__ ut,
                           const NState* st) {
  const float t = (float)st->t;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    ut[i] = fmaf(t, du[i], u[i]);
}

__global__ void k_ls_control(NState* st, const float* e0, const float* et, cudaGraphConditionalHandle h) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double E0 = *e0, Et = *et;
  const bool ok = isfinite(Et) && Et <= E0 - 1e-4 * st->t * fmax(st->slope, 0.0) + 2e-6 * fabs(E0);
  if (ok) {
    cudaGraphSetConditional(h, 0u);
    return;
  }
  if (st->ls_it >= st->ls_max) {  // no acceptable step: stop the solve
    st->apply = 0;
    st->done = 1;
    st->status = FOLGB_ERR_NOT_CONVERGED;
    cudaGraphSetConditional(h, 0u);
    return;
  }
  st->t *= 0.5;
  st->ls_it += 1;
  st->ls_halvings += 1;
  cudaGraphSetConditional(h, 1u);
}

struct NewtonWS {
  void* asm_ws;
  size_t asm_bytes;
  void* kry_ws;
  size_t kry_bytes;
  void* loss_ws;  // line search: energy evaluations
  size_t loss_bytes;
  float *r, *rhs, *du, *vals, *dinv;
  float *ut, *energy;  // line search: trial dofs, energies E(u) and E(u + t du)
  int* ls_status;
  NState* st;
  double* part;
  unsigned* counter;
  double* hist;
};

static size_t layout_newton(const folgb_plan* p, int vector_bits, int hist_cap, int line_search, void* base,
                            size_t cap, NewtonWS* w) {
  Bump bp(base, cap);
  const size_t n = (size_t)p->ndof * p->N;
  NewtonWS t;
  t.asm_bytes = folgb_workspace_bytes(p, FOLGB_OP_ASSEMBLE, 1);
  t.asm_ws = bp.take<char>(t.asm_bytes);
  t.kry_bytes = vector_bits == 64 ? krylov64_workspace_bytes(p) : pcg_workspace_bytes(p);
  t.kry_ws = bp.take<char>(t.kry_bytes);
  t.r = bp.take<float>(n);
  t.rhs = bp.take<float>(n);
  t.du = bp.take<float>(n);
  t.vals = bp.take<float>((size_t)p->nnz);
  t.dinv = bp.take<float>(n);
  t.st = bp.take<NState>(1);
  t.part = bp.take<double>(kNewtonBlocks);
  t.counter = bp.take<unsigned>(4);
  t.hist = bp.take<double>((size_t)4 * hist_cap);
  t.loss_bytes = line_search ? folgb_workspace_bytes(p, FOLGB_OP_LOSS_ADJOINT, 1) : 0;
  t.loss_ws = line_search ? bp.take<char>(t.loss_bytes) : nullptr;
  t.ut = line_search ? bp.take<float>(n) : nullptr;
  t.energy = bp.take<float>(2);
  t.ls_status = bp.take<int>(1);
  if (w) *w = t;
  return align_up(bp.off);
}

}  // namespace folgb

extern "C" size_t folgb_newton_workspace_bytes(const folgb_plan* p, const folgb_newton_settings* s) {
  if (!p || !s || !p->has_csr || s->load_steps <= 0 || s->max_iterations <= 0) return 0;
  return layout_newton(p, s->vector_bits, s->load_steps * s->max_iterations, s->line_search, nullptr, 0, nullptr);
}

extern "C" int folgb_newton(const folgb_plan* p, const float* control, float* dofs, const folgb_newton_settings* s,
                            folgb_newton_info* info, double* history, int32_t* device_status, void* workspace,
                            size_t workspace_bytes, void* stream) {
  if (!p || !control || !dofs || !s) return FOLGB_ERR_INVALID_ARGUMENT;
  if (!p->has_csr) return FOLGB_ERR_NO_PATTERN;
  if (s->load_steps <= 0 || s->max_iterations <= 0 || s->krylov_maxiter <= 0 || !(s->krylov_rtol >= 0.0) ||
      !(s->abs_tol >= 0.0) || !(s->rel_tol >= 0.0) || (s->vector_bits != 32 && s->vector_bits != 64) ||
      (s->krylov_method != FOLGB_KRYLOV_CG && s->krylov_method != FOLGB_KRYLOV_BICGSTAB) ||
      (s->line_search != 0 && s->line_search != 1) ||
      (s->line_search && (s->line_search_max_halvings < 0 || p->phys.loss_exponent != 1.0)))
    return FOLGB_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  FOLGB_CUDA_TRY(cudaStreamIsCapturing(st, &cap));
  // the solve synchronises at its end; kernel tracing would record host events
  if (cap != cudaStreamCaptureStatusNone || trace_active()) return FOLGB_ERR_INVALID_ARGUMENT;
  const int hist_cap = s->load_steps * s->max_iterations;
  NewtonWS w;
  const size_t need = layout_newton(p, s->vector_bits, hist_cap, s->line_search, workspace, workspace_bytes, &w);
  if (!workspace || workspace_bytes < need) return FOLGB_ERR_WORKSPACE;
  const int64_t n = (int64_t)p->ndof * p->N;
  const int solver = s->krylov_method == FOLGB_KRYLOV_CG ? SOLVER_CG : SOLVER_BICGSTAB;
  int vb = (int)((n + 255) / 256);
  if (vb > kNewtonBlocks) vb = kNewtonBlocks;
  int nb = (int)((p->N + 255) / 256);
  if (nb > kNewtonBlocks) nb = kNewtonBlocks;

  NState init{};
  init.abs2 = s->abs_tol * s->abs_tol;
  init.rel2 = s->rel_tol * s->rel_tol;
  init.steps = s->load_steps;
  init.maxit = s->max_iterations;
  init.status = FOLGB_OK;
  init.t = 1.0;
  init.ls_max = s->line_search_max_halvings;

  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cs = nullptr;
  int rc = FOLGB_OK;
  cudaGraphConditionalHandle loop{};
  cudaGraphNodeParams np{};
  if (cudaGraphCreate(&g, 0) != cudaSuccess || cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess ||
      cudaGraphConditionalHandleCreate(&loop, g, 1u, cudaGraphCondAssignDefault) != cudaSuccess) {
    rc = FOLGB_ERR_CUDA;
  } else {
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = loop;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np) != cudaSuccess ||
        cudaStreamBeginCaptureToGraph(cs, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed) != cudaSuccess)
      rc = FOLGB_ERR_CUDA;
  }
  // the element energy of dofs-like array v into *e (the plan's loss, no gradients)
  auto energy = [&](const float* v, float* e) {
    return folgb_loss_adjoint(p, 1, control, 0, v, n, 0, e, nullptr, nullptr, w.ls_status, w.loss_ws, w.loss_bytes,
                              cs);
  };
  if (rc == FOLGB_OK) {
    KScalars* ksc = nullptr;
    k_newton_bc<<<nb, 256, 0, cs>>>(p->N, p->ndof, p->d_dmask, p->d_dval, dofs, w.st);
    rc = folgb_assemble(p, control, dofs, 0, w.r, w.vals, w.dinv, device_status, w.asm_ws, w.asm_bytes, cs);
    if (rc == FOLGB_OK && s->line_search) rc = energy(dofs, w.energy);
    if (rc == FOLGB_OK) {
      k_newton_norm<<<vb, 256, 0, cs>>>(n, w.r, w.rhs, w.part, w.counter, &w.st->rn2);
      rc = s->vector_bits == 64
               ? krylov_solve<double>(p, solver, w.vals, w.dinv, w.rhs, w.du, s->krylov_rtol, s->krylov_maxiter,
                                      s->check_every, nullptr, nullptr, w.kry_ws, w.kry_bytes, cs, &ksc)
               : krylov_solve<float>(p, solver, w.vals, w.dinv, w.rhs, w.du, s->krylov_rtol, s->krylov_maxiter,
                                     s->check_every, nullptr, nullptr, w.kry_ws, w.kry_bytes, cs, &ksc);
    }
    if (rc == FOLGB_OK) {
      k_newton_norm<<<vb, 256, 0, cs>>>(n, w.du, nullptr, w.part, w.counter + 1, &w.st->dn2);
      if (s->line_search) {
        k_newton_dot<<<vb, 256, 0, cs>>>(n, w.rhs, w.du, w.part, w.counter + 2, &w.st->slope);
        k_ls_direction<<<vb, 256, 0, cs>>>(n, w.rhs, w.dinv, w.du, w.st, ksc);
        k_newton_dot<<<vb, 256, 0, cs>>>(n, w.rhs, w.du, w.part, w.counter + 2, &w.st->slope);
      }
      k_newton_control<<<1, 32, 0, cs>>>(w.st, ksc, w.hist, hist_cap);
      if (cudaGetLastError() != cudaSuccess) rc = FOLGB_ERR_CUDA;
    }
    if (rc == FOLGB_OK && s->line_search) {
      // nested WHILE node: trial step, its energy, accept or halve
      cudaStreamCaptureStatus bcst = cudaStreamCaptureStatusNone;
      cudaGraph_t body = nullptr;
      const cudaGraphNode_t* deps = nullptr;
      size_t ndeps = 0;
      cudaGraphConditionalHandle ls{};
      cudaStream_t ls_stream = nullptr;
      if (cudaStreamGetCaptureInfo(cs, &bcst, nullptr, &body, &deps, nullptr, &ndeps) != cudaSuccess ||
          cudaGraphConditionalHandleCreate(&ls, body, 0u, 0u) != cudaSuccess) {
        rc = FOLGB_ERR_CUDA;
      } else {
        k_ls_arm<<<1, 32, 0, cs>>>(w.st, w.energy, ls);
        cudaGraphNodeParams lp{};
        lp.type = cudaGraphNodeTypeConditional;
        lp.conditional.handle = ls;
        lp.conditional.type = cudaGraphCondTypeWhile;
        lp.conditional.size = 1;
        cudaGraphNode_t lnode;
        if (cudaGetLastError() != cudaSuccess ||
            cudaStreamGetCaptureInfo(cs, &bcst, nullptr, &body, &deps, nullptr, &ndeps) != cudaSuccess ||
            cudaGraphAddNode(&lnode, body, deps, nullptr, ndeps, &lp) != cudaSuccess ||
            cudaStreamUpdateCaptureDependencies(cs, &lnode, nullptr, 1, cudaStreamSetCaptureDependencies) !=
                cudaSuccess ||
            cudaStreamCreateWithFlags(&ls_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamBeginCaptureToGraph(ls_stream, lp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeRelaxed) != cudaSuccess) {
          rc = FOLGB_ERR_CUDA;
        } else {
          k_ls_trial<<<vb, 256, 0, ls_stream>>>(n, dofs, w.du, w.ut, w.st);
          int erc = folgb_loss_adjoint(p, 1, control, 0, w.ut, n, 0, w.energy + 1, nullptr, nullptr, w.ls_status,
                                       w.loss_ws, w.loss_bytes, ls_stream);
          k_ls_control<<<1, 32, 0, ls_stream>>>(w.st, w.energy, w.energy + 1, ls);
          const bool launched = cudaGetLastError() == cudaSuccess;
          cudaGraph_t ls_out = nullptr;
          if (cudaStreamEndCapture(ls_stream, &ls_out) != cudaSuccess || !launched || erc != FOLGB_OK)
            rc = erc != FOLGB_OK ? erc : FOLGB_ERR_CUDA;
        }
        if (ls_stream) cudaStreamDestroy(ls_stream);
      }
    }
    if (rc == FOLGB_OK) {
      k_newton_update<<<vb, 256, 0, cs>>>(n, dofs, w.du, w.st);
      k_newton_loop<<<1, 32, 0, cs>>>(w.st, loop);
      if (cudaGetLastError() != cudaSuccess) rc = FOLGB_ERR_CUDA;
    }
    cudaGraph_t body_out = nullptr;
    if (cudaStreamEndCapture(cs, &body_out) != cudaSuccess && rc == FOLGB_OK) rc = FOLGB_ERR_CUDA;
  }
  if (rc == FOLGB_OK && cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) rc = FOLGB_ERR_CUDA;
  NState fin{};
  if (rc == FOLGB_OK) {
    if (cudaMemsetAsync(w.counter, 0, 4 * sizeof(unsigned), st) != cudaSuccess ||
        cudaMemcpyAsync(w.st, &init, sizeof(NState), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaGraphLaunch(exec, st) != cudaSuccess ||
        cudaMemcpyAsync(&fin, w.st, sizeof(NState), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        (history && cudaMemcpyAsync(history, w.hist, sizeof(double) * 4 * hist_cap, cudaMemcpyDeviceToHost, st) !=
                        cudaSuccess) ||
        cudaStreamSynchronize(st) != cudaSuccess)
      rc = FOLGB_ERR_CUDA;
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (g) cudaGraphDestroy(g);
  if (cs) cudaStreamDestroy(cs);
  if (rc != FOLGB_OK) {
    cudaGetLastError();
    return rc;
  }
  if (info) {
    info->newton_iterations = fin.newton_total;
    info->krylov_iterations = fin.krylov_total;
    info->last_res_norm = fin.newton_total > 0 ? std::sqrt(fin.rn2) : 0.0;
    info->last_delta_norm = fin.newton_total > 0 ? std::sqrt(fin.dn2) : 0.0;
    info->krylov_failures = fin.krylov_fail;
    info->status = fin.status;
    info->line_search_halvings = fin.ls_halvings;
  }
  return fin.status;
}
