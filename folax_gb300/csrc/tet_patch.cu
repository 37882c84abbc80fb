// Tetrahedra in patches of six: the loss + adjoint of a tet mesh whose
// consecutive groups of 6 elements each span at most 8 nodes (the 6-tet split
// of a hexahedron, as the benchmark's tet meshes are built).
//
// The reference evaluates every tetrahedron on its own and scatters its
// energy gradient into the nodal vector (fol/loss_functions/fe_loss.py:155-164,
// 283-310, mechanical_neohooke_AD.py:254-293).  The element kernel here writes
// one record per (element, node) and a gather sums them per node: 4 records
// per tetrahedron, 24 per hexahedral cell, against 8 distinct nodes.  The patch
// kernel gives one thread the 6 tetrahedra of a patch (the same element body
// for each, its node loads hitting L1 after the first), sums their node
// results per patch node in a shared-memory column of its own in element
// order, and writes 8 records per patch (3 unpadded floats with element
// controls, else the element path's padded record); the gather then sums each
// node's patch records in ascending patch order.  A third of the records, a
// quarter of the record bytes; every sum in a fixed order (deterministic, no
// atomics).
//
// Tables (built once per mesh): per patch the local node (0..7, first
// appearance order) of each of its 24 tet corners, 4 bits each; and the node
// -> (corner, patch) incidence of the patch records.
#include <algorithm>
#include <type_traits>
#include <vector>

#include "element_body.cuh"

using namespace folgb;

namespace folgb {

int build_tet_patches(folgb_plan* p, const std::vector<int>& conn) {
  p->n_patches = 0;
  if (p->etype != FOLGB_TET4 || p->E == 0 || p->E % kPatchTets) return FOLGB_OK;
  const int64_t P = p->E / kPatchTets, N = p->N;
  if (P * kPatchNodes > INT32_MAX) return FOLGB_OK;  // int32 record indices
  std::vector<uint4> local((size_t)P);
  std::vector<int> pnode((size_t)P * kPatchNodes, -1);
  for (int64_t g = 0; g < P; ++g) {
    int ids[kPatchNodes];
    int n = 0;
    unsigned w[3] = {0u, 0u, 0u};
    for (int t = 0; t < kPatchTets; ++t)
      for (int a = 0; a < 4; ++a) {
        const int node = conn[(size_t)(g * kPatchTets + t) * 4 + a];
        int j = 0;
        while (j < n && ids[j] != node) ++j;
        if (j == n) {
          if (n == kPatchNodes) return FOLGB_OK;  // a group on more than 8 nodes: no patches
          ids[n++] = node;
        }
        w[t / 2] |= (unsigned)j << (16 * (t % 2) + 4 * a);
      }
    local[(size_t)g] = make_uint4(w[0], w[1], w[2], 0u);
    for (int j = 0; j < n; ++j) pnode[(size_t)g * kPatchNodes + j] = ids[j];
  }
  // node -> record indices corner * P + patch, ascending patch (a counting sort)
  std::vector<int> ptr((size_t)N + 1, 0);
  for (size_t k = 0; k < pnode.size(); ++k)
    if (pnode[k] >= 0) ptr[(size_t)pnode[k] + 1]++;
  for (int64_t n = 0; n < N; ++n) ptr[(size_t)n + 1] += ptr[(size_t)n];
  std::vector<int> slot((size_t)ptr[(size_t)N]);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int64_t g = 0; g < P; ++g)
    for (int j = 0; j < kPatchNodes; ++j) {
      const int node = pnode[(size_t)g * kPatchNodes + j];
      if (node >= 0) slot[(size_t)fill[(size_t)node]++] = (int)((int64_t)j * P + g);
    }
  int maxinc = 0;
  for (int64_t n = 0; n < N; ++n) maxinc = std::max(maxinc, ptr[(size_t)n + 1] - ptr[(size_t)n]);
  const int pad = maxinc <= 4 ? 4 : (maxinc <= 8 ? 8 : 0);
  std::vector<int> padded;
  if (pad) {
    padded.assign((size_t)N * pad, -1);
    for (int64_t n = 0; n < N; ++n)
      for (int k = ptr[(size_t)n]; k < ptr[(size_t)n + 1]; ++k)
        padded[(size_t)n * pad + (k - ptr[(size_t)n])] = slot[(size_t)k];
  }
  auto upload = [](auto** dst, const auto& v) -> int {
    using T = typename std::decay_t<decltype(v)>::value_type;
    const size_t n = v.empty() ? 1 : v.size();
    FOLGB_CUDA_TRY(cudaMalloc((void**)dst, n * sizeof(T)));
    if (!v.empty()) FOLGB_CUDA_TRY(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return FOLGB_OK;
  };
  int rc;
  if ((rc = upload(&p->d_patch_local, local)) || (rc = upload(&p->d_patch_inc_ptr, ptr)) ||
      (rc = upload(&p->d_patch_inc_slot, slot)) || (pad && (rc = upload(&p->d_patch_inc_padded, padded))))
    return rc;
  p->patch_pad = pad;
  p->n_patches = P;
  return FOLGB_OK;
}

void free_tet_patches(folgb_plan* p) {
  void* ptrs[] = {p->d_patch_local, p->d_patch_inc_ptr, p->d_patch_inc_slot, p->d_patch_inc_padded};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  p->d_patch_local = nullptr;
  p->d_patch_inc_ptr = p->d_patch_inc_slot = p->d_patch_inc_padded = nullptr;
  p->n_patches = 0;
}

namespace {

constexpr int kPatchBlock = 256;

// One thread per (instance, patch); the grid is (instances, patch blocks) so
// the instances of one patch range share the mesh loads in L2, and a block
// takes `tiles` consecutive ranges of 256 patches.
template <int PH, int NP>
__global__ void __launch_bounds__(kPatchBlock, NP == 1 ? 4 : 2) k_tet_patch(const VecArgs A, const uint4* __restrict__ plocal,
                                                              const int64_t P, const int tiles) {
  __shared__ GPTable gp;
  __shared__ float wsum[32];
  __shared__ unsigned wcount;
  __shared__ float4 acc[kPatchNodes][kPatchBlock];  // a column of 8 node sums per thread
  pdl_launch_dependents();
  if constexpr (NP == 0) load_gp_table(gp, A.gp);
  if (threadIdx.x == 0) wcount = 0u;
  __syncthreads();
  const int b = blockIdx.x, blk = blockIdx.y, nblk = gridDim.y;
  float energy = 0.f;
  int bad = 0;
  for (int k = 0; k < tiles; ++k) {
    const int64_t pt = ((int64_t)blk * tiles + k) * kPatchBlock + threadIdx.x;
    if (pt >= P) break;
#pragma unroll
    for (int j = 0; j < kPatchNodes; ++j) acc[j][threadIdx.x] = make_float4(0.f, 0.f, 0.f, 0.f);
    const uint4 L = __ldg(plocal + pt);
#pragma unroll 1
    for (int t = 0; t < kPatchTets; ++t) {
      const unsigned w = (t < 2 ? L.x : (t < 4 ? L.y : L.z)) >> (16 * (t & 1));
      elem_vector_body_to<FOLGB_TET4, PH, MODE_LOSS, NP>(
          A, gp, b, (int64_t)kPatchTets * pt + t, energy, bad, [&](int a, const float (&v)[4]) {
            float4& s = acc[(w >> (4 * a)) & 7u][threadIdx.x];
            float4 c = s;
            c.x += v[0];
            c.y += v[1];
            c.z += v[2];
            c.w += v[3];
            s = c;
          });
    }
    // records [b][corner][P], local-node-major like the element records
#pragma unroll
    for (int j = 0; j < kPatchNodes; ++j) {
      const float4 c = acc[j][threadIdx.x];
      const float v[4] = {c.x, c.y, c.z, c.w};
      store_record(A, (((int64_t)b * kPatchNodes + j) * P + pt) * A.rec, v);
    }
  }
  finish_loss_warp(energy, bad, A, b, wsum, &wcount, blk, nblk);
}

template <int PH>
int launch_typed(const folgb_plan* p, const VecArgs& A0, int B, int64_t nb, int tiles, cudaStream_t s) {
  VecArgs A = A0;
  A.rec = tet_patch_record(p);
  with_const_gp<FOLGB_TET4>(p, [&](auto np) {
    constexpr int NP = decltype(np)::value;
    k_tet_patch<PH, NP><<<dim3((unsigned)B, (unsigned)nb), kPatchBlock, 0, s>>>(A, p->d_patch_local, p->n_patches,
                                                                              tiles);
  });
  return 1;
}

}  // namespace

int launch_tet_patch(const folgb_plan* p, const VecArgs& A, int B, cudaStream_t s) {
  // kernel_variant 1 (the generic per-element loop) keeps one record per element node
  if (p->n_patches <= 0 || p->phys.kernel_variant == 1 || p->ndof != 3 || B > 65535) return 0;
  if (p->physics != FOLGB_ELASTIC && p->physics != FOLGB_NEOHOOKE && p->physics != FOLGB_SAINT_VENANT &&
      p->physics != FOLGB_NEOHOOKE_SPLIT)
    return 0;
  // patch ranges per block: up to 16 while the launch keeps 8 waves of 4
  // blocks per SM (the element kernel's rule)
  const int64_t nb0 = (p->n_patches + kPatchBlock - 1) / kPatchBlock;
  int tiles = 1;
  while (tiles < 16 && ((nb0 + 2 * tiles - 1) / (2 * tiles)) * B >= (int64_t)32 * num_sms()) tiles *= 2;
  const int64_t nb = (nb0 + tiles - 1) / tiles;
  if (nb > 65535) return 0;
  int rc = 0;
  trace_begin(KID_ELEM_LOSS, s);
  switch (p->physics) {
    case FOLGB_ELASTIC: rc = launch_typed<FOLGB_ELASTIC>(p, A, B, nb, tiles, s); break;
    case FOLGB_NEOHOOKE: rc = launch_typed<FOLGB_NEOHOOKE>(p, A, B, nb, tiles, s); break;
    case FOLGB_SAINT_VENANT: rc = launch_typed<FOLGB_SAINT_VENANT>(p, A, B, nb, tiles, s); break;
    case FOLGB_NEOHOOKE_SPLIT: rc = launch_typed<FOLGB_NEOHOOKE_SPLIT>(p, A, B, nb, tiles, s); break;
  }
  trace_end(KID_ELEM_LOSS, s);
  if (rc && cudaGetLastError() != cudaSuccess) return -FOLGB_ERR_CUDA;
  return rc;
}

}  // namespace folgb
