// Many parametric instances with uneven meshes in one persistent launch.
//
// The instances are concatenated into one disconnected mesh (global node ids)
// whose tables are an ordinary plan; per-instance offset tables add
//   tiles: (instance, first element, count) with every tile inside one
//          instance, so each tile's energy partial belongs to one instance;
//   node_inst / elem_inst: instance of each node / element (gradient scale).
// A persistent kernel (a few CTAs per SM) walks the tiles; the CTA that
// finishes last sums each instance's tile partials in tile order (a
// deterministic segmented reduction) into L_i and the gradient scale
// p L_i^(p-1) / I.  The reference batches a single mesh only
// (fol/loss_functions/fe_loss.py:250-262); this path has no counterpart there.
#include <algorithm>
#include <vector>

#include "element_body.cuh"

using namespace folgb;

struct folgb_batch_plan {
  folgb_plan* mesh = nullptr;
  int32_t I = 0;
  int64_t ntiles = 0;
  int64_t max_tiles = 0;  // tiles at the smallest tile size the autotuner tries
  int tile = 0;
  std::vector<int64_t> eoff;  // host copy of the instance element offsets
  int64_t* d_tile_start = nullptr;
  int* d_tile_count = nullptr;
  int* d_tile_off = nullptr;   // [I+1] tile range of each instance
  int* d_node_inst = nullptr;
  int* d_elem_inst = nullptr;
};

namespace folgb {
int check_physics(const folgb_physics* phys, int& nen, int& dim, int& ndof);

struct BatchArgs {
  int64_t ntiles;
  const int64_t* tile_start;
  const int* tile_count;
  const int* tile_off;
  int I;
};

// Each warp writes its own energy partial of every tile it works on
// (partials[t][warp]), so a tile needs no block barrier; the last block sums
// an instance's partials in (tile, warp) order.
constexpr int kBatchWarps = 8;  // 256 threads

template <int ET, int PH, int NP = 0>
__global__ void __launch_bounds__(kBatchWarps * 32) k_batch_loss(const VecArgs A, const BatchArgs T) {
  __shared__ GPTable gp;
  __shared__ bool last;
  if constexpr (NP == 0) load_gp_table(gp, A.gp);  // a compile-time rule needs no table
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int bad = 0;
  for (int64_t t = blockIdx.x; t < T.ntiles; t += gridDim.x) {
    const int64_t e0 = T.tile_start[t];
    const int cnt = T.tile_count[t];
    float energy = 0.f;
    for (int k = threadIdx.x; k < cnt; k += blockDim.x)
      elem_vector_body<ET, PH, MODE_LOSS, NP>(A, gp, 0, e0 + k, energy, bad);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) energy += __shfl_xor_sync(0xffffffffu, energy, o);
    if (lane == 0) A.partials[t * kBatchWarps + warp] = energy;
  }
  __threadfence();  // this warp's partials are visible before the block is counted
  report_bad(bad, A.status);  // a block barrier
  if (threadIdx.x == 0) {
    unsigned prev = atomicAdd(A.counters, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const volatile float* pv = A.partials;
  const float p = A.exponent;
  for (int i = threadIdx.x; i < T.I; i += blockDim.x) {
    float L = 0.f;
    for (int t = T.tile_off[i]; t < T.tile_off[i + 1]; ++t)
#pragma unroll
      for (int w = 0; w < kBatchWarps; ++w) L += pv[t * kBatchWarps + w];
    const float Lp = (p == 1.f) ? L : powf(L, p);
    A.losses[i] = Lp;
    A.scale[i] = (p == 1.f) ? A.inv_batch : p * powf(L, p - 1.f) * A.inv_batch;
    if (!isfinite(Lp) && A.status) atomicOr(A.status, 1 << FOLGB_ERR_NAN);
  }
  if (threadIdx.x == 0) A.counters[0] = 0u;
}

struct BatchWS {
  float* g;
  int rec;
  float* partials;
  unsigned* counters;
  float* scale;
};

static size_t layout_batch(const folgb_batch_plan* bp, void* base, size_t cap, BatchWS* w) {
  const folgb_plan* p = bp->mesh;
  Bump b(base, cap);
  BatchWS t;
  t.rec = loss_record(p);
  t.g = b.take<float>((size_t)p->E * p->nen * t.rec);
  t.partials = b.take<float>((size_t)std::max(bp->ntiles, bp->max_tiles) * kBatchWarps);
  t.counters = b.take<unsigned>(1);
  t.scale = b.take<float>((size_t)bp->I);
  if (w) *w = t;
  return align_up(b.off);
}

template <class T>
static int upload_vec(T** dst, const std::vector<T>& v) {
  FOLGB_CUDA_TRY(cudaMalloc((void**)dst, std::max<size_t>(1, v.size()) * sizeof(T)));
  if (!v.empty()) FOLGB_CUDA_TRY(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return FOLGB_OK;
}

// tile sizes the autotuner tries (elements per tile, every tile inside one instance)
constexpr int kBatchTiles[] = {256, 512, 1024, 2048, 4096};
constexpr int kBatchTileCount = 5;

static int64_t count_tiles(const std::vector<int64_t>& eoff, int tile) {
  int64_t n = 0;
  for (size_t i = 0; i + 1 < eoff.size(); ++i) n += (eoff[i + 1] - eoff[i] + tile - 1) / tile;
  return n;
}

// (re)builds the tile tables of the plan for `tile` elements per tile
static int build_tiles(folgb_batch_plan* bp, int tile) {
  std::vector<int64_t> tstart;
  std::vector<int> tcount, toff(bp->I + 1, 0);
  for (int i = 0; i < bp->I; ++i) {
    toff[i] = (int)tstart.size();
    for (int64_t e = bp->eoff[i]; e < bp->eoff[i + 1]; e += tile) {
      tstart.push_back(e);
      tcount.push_back((int)std::min<int64_t>(tile, bp->eoff[i + 1] - e));
    }
  }
  toff[bp->I] = (int)tstart.size();
  void* old[] = {bp->d_tile_start, bp->d_tile_count, bp->d_tile_off};
  for (void* q : old)
    if (q) cudaFree(q);
  bp->d_tile_start = nullptr;
  bp->d_tile_count = nullptr;
  bp->d_tile_off = nullptr;
  bp->tile = tile;
  bp->ntiles = (int64_t)tstart.size();
  int rc;
  if ((rc = upload_vec(&bp->d_tile_start, tstart)) || (rc = upload_vec(&bp->d_tile_count, tcount)) ||
      (rc = upload_vec(&bp->d_tile_off, toff)))
    return rc;
  return FOLGB_OK;
}

}  // namespace folgb

extern "C" int folgb_batch_plan_destroy(folgb_batch_plan* bp) {
  if (!bp) return FOLGB_OK;
  folgb_plan_destroy(bp->mesh);
  void* ptrs[] = {bp->d_tile_start, bp->d_tile_count, bp->d_tile_off, bp->d_node_inst, bp->d_elem_inst};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  delete bp;
  return FOLGB_OK;
}

extern "C" int folgb_batch_plan_create(folgb_batch_plan** out, const folgb_physics* phys, int32_t I,
                                       const int64_t* eoff, const int64_t* noff, const int64_t* conn,
                                       const double* xyz, const int64_t* dirichlet_dofs,
                                       const double* dirichlet_values, int64_t num_dirichlet,
                                       int32_t elements_per_tile) {
  if (!out || I <= 0 || !eoff || !noff || !conn || !xyz) return FOLGB_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int nen, dim, ndof;
  int rc = check_physics(phys, nen, dim, ndof);
  if (rc) return rc;
  if (eoff[0] != 0 || noff[0] != 0) return FOLGB_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < I; ++i)
    if (eoff[i + 1] <= eoff[i] || noff[i + 1] <= noff[i]) return FOLGB_ERR_INVALID_ARGUMENT;
  const int64_t E = eoff[I], N = noff[I];
  // local -> global node ids
  std::vector<int64_t> gconn((size_t)E * nen);
  for (int i = 0; i < I; ++i) {
    const int64_t nloc = noff[i + 1] - noff[i];
    for (int64_t e = eoff[i]; e < eoff[i + 1]; ++e)
      for (int a = 0; a < nen; ++a) {
        int64_t v = conn[e * nen + a];
        if (v < 0 || v >= nloc) return FOLGB_ERR_INVALID_ARGUMENT;
        gconn[e * nen + a] = v + noff[i];
      }
  }
  folgb_batch_plan* bp = new folgb_batch_plan();
  rc = folgb_plan_create(&bp->mesh, phys, gconn.data(), E, xyz, N, dirichlet_dofs, dirichlet_values, num_dirichlet,
                         0);
  if (rc) {
    delete bp;
    return rc;
  }
  const int tile = elements_per_tile > 0 ? elements_per_tile : 1024;
  bp->I = I;
  bp->eoff.assign(eoff, eoff + I + 1);
  bp->max_tiles = std::max(count_tiles(bp->eoff, kBatchTiles[0]), count_tiles(bp->eoff, tile));
  std::vector<int> node_inst(N), elem_inst(E);
  for (int i = 0; i < I; ++i) {
    for (int64_t n = noff[i]; n < noff[i + 1]; ++n) node_inst[n] = i;
    for (int64_t e = eoff[i]; e < eoff[i + 1]; ++e) elem_inst[e] = i;
  }
  if ((rc = build_tiles(bp, tile)) || (rc = upload_vec(&bp->d_node_inst, node_inst)) ||
      (rc = upload_vec(&bp->d_elem_inst, elem_inst))) {
    folgb_batch_plan_destroy(bp);
    return rc;
  }
  *out = bp;
  return FOLGB_OK;
}

extern "C" size_t folgb_batch_workspace_bytes(const folgb_batch_plan* bp) {
  if (!bp) return 0;
  return layout_batch(bp, nullptr, 0, nullptr);
}

extern "C" int folgb_batch_loss_adjoint(const folgb_batch_plan* bp, const float* control, const float* dofs,
                                        int32_t apply_dirichlet, float* losses, float* dloss_ddofs,
                                        float* dloss_dcontrol, int32_t* device_status, void* workspace,
                                        size_t workspace_bytes, void* stream) {
  if (!bp || !control || !dofs || !losses) return FOLGB_ERR_INVALID_ARGUMENT;
  // a tile table that could not be (re)built leaves the plan unusable
  if (!bp->d_tile_start || !bp->d_tile_count || !bp->d_tile_off) return FOLGB_ERR_CUDA;
  const folgb_plan* p = bp->mesh;
  BatchWS w;
  size_t need = layout_batch(bp, workspace, workspace_bytes, &w);
  if (!workspace || workspace_bytes < need) return FOLGB_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  FOLGB_CUDA_TRY(cudaMemsetAsync(w.counters, 0, sizeof(unsigned), s));
  const bool elem_ctrl = p->ctrl_layout == FOLGB_CONTROL_ELEMENT;
  VecArgs A;
  A.E = p->E;
  A.N = p->N;
  A.conn = p->d_conn;
  A.xyz4 = p->d_xyz4;
  A.gp = p->d_gp;
  A.ctrl = control;
  A.ctrl_stride = 0;
  A.dofs = dofs;
  A.dofs_stride = 0;
  A.dmask = p->d_dmask;
  A.elem_bc = p->d_elem_bc;
  A.k0 = p->d_k0;
  A.dval = p->d_dval;
  A.apply_dirichlet = apply_dirichlet;
  A.ctrl_layout = p->ctrl_layout;
  A.mat = p->mat;
  A.g = w.g;
  A.rec = w.rec;
  A.dctrl_elem = elem_ctrl ? dloss_dcontrol : nullptr;
  A.partials = w.partials;
  A.counters = w.counters;
  A.losses = losses;
  A.scale = w.scale;
  A.exponent = (float)p->phys.loss_exponent;
  A.inv_batch = 1.f / (float)bp->I;
  A.status = device_status;
  BatchArgs T{bp->ntiles, bp->d_tile_start, bp->d_tile_count, bp->d_tile_off, bp->I};
  int64_t grid = std::min<int64_t>(bp->ntiles, (int64_t)num_sms() * 4);
  int rc = dispatch(p->etype, p->physics, [&](auto tag) -> int {
    constexpr int ET = decltype(tag)::ET, PH = decltype(tag)::PH;
    trace_begin(KID_BATCH_LOSS, s);
    with_const_gp<ET>(p, [&](auto np) {
      k_batch_loss<ET, PH, decltype(np)::value><<<(unsigned)grid, 256, 0, s>>>(A, T);
    });
    trace_end(KID_BATCH_LOSS, s);
    FOLGB_LAUNCH_CHECK();
    return (int)FOLGB_OK;
  });
  if (rc) return rc;
  if (dloss_ddofs || dloss_dcontrol) {
    rc = launch_gather(p, 1, w.g, w.rec, elem_ctrl ? 0 : 1, w.scale, dloss_ddofs, 0,
                       elem_ctrl ? nullptr : dloss_dcontrol, 0, elem_ctrl ? dloss_dcontrol : nullptr,
                       (elem_ctrl && p->phys.loss_exponent != 1.0) ? 1 : 0, s, bp->d_node_inst, bp->d_elem_inst);
  }
  return rc;
}

// Times the batched loss + adjoint with each tile size of kBatchTiles (2
// warm-up and `repeats` timed calls each, CUDA events on the stream, the
// flush buffer, if given, overwritten before every timed call outside its
// events) and keeps the fastest tile size in the plan.  Synchronises the
// stream; the tile tables are rebuilt between candidates, so no other work
// may use the plan meanwhile.
extern "C" int folgb_batch_autotune(folgb_batch_plan* bp, const float* control, const float* dofs,
                                    int32_t apply_dirichlet, float* losses, float* dloss_ddofs,
                                    float* dloss_dcontrol, int32_t* device_status, void* workspace,
                                    size_t workspace_bytes, int32_t repeats, void* flush_buffer, size_t flush_bytes,
                                    void* stream, int32_t* chosen_tile, float* ms_per_candidate,
                                    int32_t max_candidates) {
  if (!bp || !chosen_tile || !control || !dofs || !losses) return FOLGB_ERR_INVALID_ARGUMENT;
  if (!workspace || workspace_bytes < layout_batch(bp, nullptr, 0, nullptr)) return FOLGB_ERR_WORKSPACE;
  if (repeats < 1) repeats = 1;
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  FOLGB_CUDA_TRY(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return FOLGB_ERR_CUDA;
  }
  const int start_tile = bp->tile;
  int rc = FOLGB_OK, best = -1;
  float best_ms = 0.f;
  auto call = [&]() {
    return folgb_batch_loss_adjoint(bp, control, dofs, apply_dirichlet, losses, dloss_ddofs, dloss_dcontrol,
                                    device_status, workspace, workspace_bytes, stream);
  };
  for (int c = 0; c < kBatchTileCount && !rc; ++c) {
    if (cudaStreamSynchronize(s) != cudaSuccess) {
      rc = FOLGB_ERR_CUDA;
      break;
    }
    if ((rc = build_tiles(bp, kBatchTiles[c]))) break;
    for (int w = 0; w < 2 && !rc; ++w) rc = call();
    float total = 0.f;
    for (int r = 0; r < repeats && !rc; ++r) {
      if (flush_buffer && flush_bytes && cudaMemsetAsync(flush_buffer, r & 0xff, flush_bytes, s) != cudaSuccess) {
        rc = FOLGB_ERR_CUDA;
        break;
      }
      if (cudaEventRecord(e0, s) != cudaSuccess) rc = FOLGB_ERR_CUDA;
      if (!rc) rc = call();
      if (!rc && (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess))
        rc = FOLGB_ERR_CUDA;
      float ms = 0.f;
      if (!rc && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = FOLGB_ERR_CUDA;
      total += ms;
    }
    if (rc) break;
    const float ms = total / (float)repeats;
    if (ms_per_candidate && c < max_candidates) ms_per_candidate[c] = ms;
    if (best < 0 || ms < best_ms) {
      best = c;
      best_ms = ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // keep the fastest (or, after a failure, the tile size the plan had)
  if (cudaStreamSynchronize(s) != cudaSuccess && !rc) rc = FOLGB_ERR_CUDA;
  const int keep = (!rc && best >= 0) ? kBatchTiles[best] : start_tile;
  const int rc2 = build_tiles(bp, keep);
  if (!rc) rc = rc2;
  if (!rc) *chosen_tile = keep;
  return rc;
}
