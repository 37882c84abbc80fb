// Internal declarations shared by the folgb translation units.
//
// Data layout in HBM (built once per mesh by folgb_plan_create):
//   conn      int32 [E][nen]          element -> node ids (16/32-byte rows)
//   xyz4      float4[N]               node coordinates padded to 16 bytes
//   inc_ptr   int32 [N+1]             node -> incident (element, local node) (CSR)
//   inc_slot  int32 [E*nen]           record index a*E + e, ascending e per node
//   element results ("records"): [B][nen][E] x 1/2/4 floats, local-node-major
//   dmask     uint8 [N]               bit c set if dof (node, c) is Dirichlet
//   dval      float [ndof*N]          Dirichlet value (read only where masked)
//   gp        GPTable                 Gauss points: w, N, dN/dxi (fp32)
// CSR tables (optional):
//   adj_ptr/adj   node-pair pattern (sorted neighbours, self included)
//   rowptr/colind canonical dof-level CSR (row ndof*n+c)
//   pair_row      row node of each node pair
//   pair_ptr/pair_slot  pair -> contributing element-matrix blocks,
//                       slot = (e*nen + a)*nen + b, ascending e (the segments
//                       of the deterministic reduction)
#pragma once

#include <cstdint>
#include <cstdio>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/folgb.h"

namespace folgb {

constexpr int kMaxGP = 27;
constexpr int kMaxNen = 8;

struct GPTable {
  int npts;
  int pad_[3];
  float w[kMaxGP];
  float N[kMaxGP][kMaxNen];
  float dN[kMaxGP][kMaxNen][3];
};

// Material/physics constants in the precision the kernels use.
struct MatConst {
  float lam, mu;        // elastic: D = e_gp * (lam, mu) isotropic (2-D: plane stress pair)
  float lam_f, mu_f;    // neo-Hooke: lambda = lam_f * e_gp, mu = mu_f * e_gp
  float beta, c;        // thermal conductivity nonlinearity
  float bf[3];          // body force
  int has_bf;
  int shear_ref;        // 1: reference (doubled) shear for the FE residual/tangent
  float rho_cp, dt, mbeta;  // transient thermal: rho cp, time step, material beta
  float kap_f;          // split neo-Hooke: kappa = kap_f * e_gp, mu = mu_f * e_gp
};

// Element matrix of a uniform axis-aligned box mesh in the Walsh-Hadamard basis
// of the nodal values (uniform_box.cu): the 3 x 3 block of each reflection
// parity p, coupling the modes (component 0, p^1), (1, p^2), (2, p^4).
struct BoxK {
  float k[8][3][3];
};

// Hyperelastic physics: residual B(F)^T S, tangent B^T C B + geometric stiffness.
constexpr bool is_hyperelastic(int ph) {
  return ph == FOLGB_NEOHOOKE || ph == FOLGB_SAINT_VENANT || ph == FOLGB_NEOHOOKE_SPLIT;
}

}  // namespace folgb

struct folgb_plan {
  folgb_physics phys;
  int etype, physics, nen, dim, ndof;
  int64_t E, N;
  int ctrl_layout;
  folgb::MatConst mat;
  folgb::GPTable h_gp;
  // device tables
  int* d_conn = nullptr;
  float4* d_xyz4 = nullptr;
  int* d_inc_ptr = nullptr;
  int* d_inc_slot = nullptr;
  int inc_pad = 0;          // 4 or 8 when every node has at most that many incidences, else 0
  int* d_inc_padded = nullptr;  // [N][inc_pad] incident slots, -1 padded (vector loads)
  // tetrahedra in patches of 6 consecutive elements on at most 8 nodes (the
  // 6-tet split of a hexahedron; tet_patch.cu): per patch the local node
  // (0..7) of each tet corner, 4 bits each, tet t in bits 16 (t % 2) + 4 a of
  // word t / 2; and the node -> (corner, patch) incidence of the patch records
  int64_t n_patches = 0;                // 0: no patch tables
  uint4* d_patch_local = nullptr;       // [P]
  int* d_patch_inc_ptr = nullptr;       // [N + 1]
  int* d_patch_inc_slot = nullptr;      // record indices corner * P + patch, ascending patch
  int patch_pad = 0;                    // 4 or 8 when every node has at most that many, else 0
  int* d_patch_inc_padded = nullptr;    // [N][patch_pad], -1 padded
  int hex8_variant = 0;    // sum-factorised hex8 kernel variant (autotuned)
  unsigned char* d_dmask = nullptr;
  unsigned char* d_elem_bc = nullptr;  // [E] 1 if a node of the element has a Dirichlet dof
  float* d_k0 = nullptr;               // [N] nodal material field (transient thermal k0)
  float* d_dval = nullptr;
  folgb::GPTable* d_gp = nullptr;
  std::vector<int64_t> dir_dofs;
  std::vector<double> dir_vals;
  // Element tiles of the tile-local fused loss (tiles.cu): elements grouped
  // into tiles of at most kTileElems elements and kTileNodes distinct nodes
  // (Morton order of the centroids, closed greedily); per tile its elements,
  // its distinct ("local") nodes, boundary ones first, and for each local
  // node the shared-memory records that contribute to it.
  int tiles = 0;                        // 0: no tile tables (other element types / physics)
  int64_t tile_local_nodes = 0;         // K: local node slots over all tiles
  int64_t tile_boundary_slots = 0;      // S: boundary local node slots (partial records per instance)
  int64_t tile_boundary_nodes = 0;      // NB: nodes in 0 or more than 1 tile
  int64_t tile_interior_nodes = 0;      // NI: nodes inside exactly one tile
  int* d_tile_eptr = nullptr;           // [T+1] element range of each tile (tile order)
  int* d_tile_nptr = nullptr;           // [T+1] local node range of each tile
  int* d_tile_bptr = nullptr;           // [T+1] boundary slot range of each tile (its first local nodes)
  int* d_t_elem = nullptr;              // [E] element ids in tile order, bit 31: touches a Dirichlet dof
  unsigned char* d_t_lconn = nullptr;   // [E][nen] local node ids, reference node order
  unsigned short* d_tn_pos = nullptr;   // [K][kTileRecs] record positions a*kTileElems + e_local of each
                                        // local entry, padded with kTileZeroRec
  int* d_tn_gid = nullptr;              // [K] global node id of each local node
  unsigned* d_tn_info = nullptr;        // [K] bits 16-18: the node's Dirichlet mask
  int* d_bn_node = nullptr;             // [NB] boundary nodes
  int* d_bn_ptr = nullptr;              // [NB+1] their partial slots
  int* d_bn_slot = nullptr;             // [S] slots in ascending tile order
  int* d_in_node = nullptr;             // [NI] interior nodes (rescaled when the loss exponent is not 1)
  // every element the same axis-aligned box (uniform_box.cu): the blocks of
  // its element matrix for the box kernels, box_valid 0 otherwise
  int box_valid = 0;
  folgb::BoxK box_k = {};
  // and the box mesh numbering of an nx x ny x nz grid (nodes x fastest, then
  // y, then z; the reference local node order): the one-launch grid kernel
  int box_grid = 0, box_nx = 0, box_ny = 0, box_nz = 0;
  unsigned char* d_box_layer_bc = nullptr;  // [nz + 1] node layer has a Dirichlet dof (grid kernel)

  // instantiated Krylov solve graphs of folgb_krylov_async (krylov.cu)
  void* krylov_graphs = nullptr;
  // CSR tables
  bool has_csr = false;
  int64_t P = 0, nnz = 0, rows = 0;
  int maxdeg = 0;
  int* d_adj_ptr = nullptr;
  int* d_adj = nullptr;
  int* d_rowptr = nullptr;
  int* d_colind = nullptr;
  int* d_pair_row = nullptr;
  int* d_pair_ptr = nullptr;
  int* d_pair_slot = nullptr;
};

namespace folgb {

// ---------------------------------------------------------------------------
// error helpers
// ---------------------------------------------------------------------------
#define FOLGB_CUDA_TRY(expr)                                                        \
  do {                                                                              \
    cudaError_t err__ = (expr);                                                     \
    if (err__ != cudaSuccess) {                                                     \
      fprintf(stderr, "folgb: %s failed: %s (%s:%d)\n", #expr,                      \
              cudaGetErrorString(err__), __FILE__, __LINE__);                       \
      return (int)FOLGB_ERR_CUDA;                                                      \
    }                                                                               \
  } while (0)

#define FOLGB_LAUNCH_CHECK() FOLGB_CUDA_TRY(cudaGetLastError())

inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// Simple bump allocator over a caller-provided workspace.
struct Bump {
  char* base;
  size_t cap, off = 0;
  Bump(void* b, size_t c) : base(static_cast<char*>(b)), cap(c) {}
  template <class T>
  T* take(size_t count) {
    size_t o = align_up(off);
    off = o + count * sizeof(T);
    return reinterpret_cast<T*>(base + o);
  }
  bool ok() const { return base != nullptr && off <= cap; }
};

int num_sms();

// Looks up the no-alloc scratch array on the current device (noalloc.cu).
void noalloc_prepare_current_device();

// Element tiles of the tile-local fused loss (tiles.cu).
constexpr int kTileElems = 128;  // elements per tile at most (one thread each)
constexpr int kTileNodes = 256;  // local node entries per tile at most (8-bit local ids)
constexpr int kTileRecs = 8;     // records per local node entry (one 16-byte row of positions)
constexpr int kTileZeroRec = 8 * kTileElems;  // position of the zero record padding the rows
int build_tile_tables(folgb_plan* p, const std::vector<int>& conn, const double* xyz,
                      const std::vector<unsigned char>& dmask, const std::vector<unsigned char>& elem_bc);
void free_tile_tables(folgb_plan* p);
// Tet patches (tet_patch.cu): sets n_patches and the patch tables when every
// group of 6 consecutive tetrahedra spans at most 8 nodes.
constexpr int kPatchTets = 6, kPatchNodes = 8;
int build_tet_patches(folgb_plan* p, const std::vector<int>& conn);
void free_tet_patches(folgb_plan* p);
// Uniform axis-aligned box elements (uniform_box.cu): sets box_valid and box_k.
int build_uniform_box(folgb_plan* p, const std::vector<float4>& x4, const std::vector<int>& conn,
                      const std::vector<unsigned char>& dmask);
void box_hadamard_stiffness(const double (&J)[3][3], double lam, double mu, double (&khat)[24][24]);
// most blocks per instance of the structured box grid kernel (hex8_fused.cu)
int64_t grid_blocks_max(const folgb_plan* p);

// Destroys the plan's cached Krylov solve graphs (krylov.cu).
void free_krylov_graphs(folgb_plan* p);

// Element-result records: one per (instance, element, node), [b][a][e],
// padded to 1, 2 or 4 floats so the gather reads them with one vector load.
// Components [0, ndof) hold the vector; component ndof the nodal control
// sensitivity when the loss path has one.
inline int padded_record(int n) { return n <= 1 ? 1 : (n <= 2 ? 2 : 4); }
inline int loss_record(const folgb_plan* p);
inline int residual_record(const folgb_plan* p);

// deterministic node gather of element vectors (elements.cu)
// pdl = 1: launched as a programmatic dependent of the element kernel just
// before it on the stream (its incidence loads overlap that kernel's tail).
// patches = 1: the records are the tet patch kernel's ([B][8][P], the patch
// incidence tables)
int launch_gather(const folgb_plan* p, int B, const float* g, int rec, int with_gde, const float* scale, float* out,
                  int64_t out_stride, float* dctrl, int64_t dctrl_stride, float* dctrl_elem, int rescale_elem,
                  cudaStream_t s, const int* node_inst, const int* elem_inst, int pdl = 0, int patches = 0);

// Programmatic dependent launch: the primary kernel lets the next kernel on
// the stream start early; the dependent waits for the primary's completion
// (and memory) before touching its results.  Both are no-ops without the
// launch attribute.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;"); }
__device__ __forceinline__ void pdl_wait_primary() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// ---------------------------------------------------------------------------
// Bulk asynchronous copies (TMA engine) completing on shared-memory mbarriers
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// makes the initialised barriers visible to the async (TMA) proxy
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// orders earlier generic-proxy accesses of shared memory before later async-proxy ones
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// one arrival that also announces `bytes` of transactions for the current phase
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Waits for the phase with the given parity to complete; gives up after
// about 2^22 polls (tens of milliseconds with the back-off), so a copy that
// never lands cannot hang the kernel.  Returns false if it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
  for (int i = 0; i < (1 << 22); ++i) {
    if (mbar_test_wait(bar, parity)) return true;
    if (i >= 64) __nanosleep(32);
  }
  return false;
}
// global -> shared bulk copy of `bytes` (multiple of 16; both addresses
// 16-byte aligned), completing `bytes` transactions on bar
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// ---------------------------------------------------------------------------
// element traits
// ---------------------------------------------------------------------------
template <int ET> struct ElemT;
template <> struct ElemT<FOLGB_QUAD4> { static constexpr int NEN = 4, DIM = 2; };
template <> struct ElemT<FOLGB_HEX8>  { static constexpr int NEN = 8, DIM = 3; };
template <> struct ElemT<FOLGB_TET4>  { static constexpr int NEN = 4, DIM = 3; };

// Reference derivatives dN_a/dxi_k at Gauss point q.  The linear tetrahedron
// (N = 1 - xi - eta - zeta, xi, eta, zeta; tetrahedra_3d_4.py:48-60) has the
// same gradients at every point: compile-time constants, so its Jacobian and
// dN/dx fold to differences and copies (the same values as the table's).
// Compile-time Gauss rules for the small common cases (NP points; NP = 0:
// the plan's table at run time): quad4 with the 2x2 rule (NP 4) and tet4
// with the 1-point rule (NP 1), in the reference's point order
// (quadrilateral_2d_4.py:22-31, tetrahedra_3d_4.py:16-20) and with the table's
// values (computed in double, rounded to float), so loops over them unroll
// into constants.
template <int ET, int NP> struct GPc;
template <> struct GPc<FOLGB_QUAD4, 4> {
  static constexpr double g = 0.57735026918962576451;  // 1/sqrt(3)
  __device__ static constexpr double sx(int a) { return (a == 1 || a == 2) ? 1.0 : -1.0; }
  __device__ static constexpr double sy(int a) { return a >= 2 ? 1.0 : -1.0; }
  __device__ static constexpr float w(int) { return 1.f; }
  __device__ static constexpr float N(int q, int a) {
    return (float)(0.25 * (1.0 + sx(a) * (sx(q) * g)) * (1.0 + sy(a) * (sy(q) * g)));
  }
  __device__ static constexpr float dN(int q, int a, int k) {
    return k == 0 ? (float)(0.25 * sx(a) * (1.0 + sy(a) * (sy(q) * g)))
                  : (k == 1 ? (float)(0.25 * sy(a) * (1.0 + sx(a) * (sx(q) * g))) : 0.f);
  }
};
template <> struct GPc<FOLGB_TET4, 1> {
  __device__ static constexpr float w(int) { return (float)(1.0 / 6.0); }
  __device__ static constexpr float N(int, int) { return 0.25f; }
  __device__ static constexpr float dN(int, int a, int k) { return a == 0 ? -1.f : (a - 1 == k ? 1.f : 0.f); }
};

template <int ET, int NP = 0>
__device__ __forceinline__ float dN_at(const GPTable& gp, int q, int a, int k) {
  if constexpr (NP > 0) return GPc<ET, NP>::dN(q, a, k);
  else if constexpr (ET == FOLGB_TET4) return a == 0 ? -1.f : (a - 1 == k ? 1.f : 0.f);
  else return gp.dN[q][a][k];
}
template <int ET, int NP = 0>
__device__ __forceinline__ float gp_w(const GPTable& gp, int q) {
  if constexpr (NP > 0) return GPc<ET, NP>::w(q);
  else return gp.w[q];
}
template <int ET, int NP = 0>
__device__ __forceinline__ float gp_N(const GPTable& gp, int q, int a) {
  if constexpr (NP > 0) return GPc<ET, NP>::N(q, a);
  else return gp.N[q][a];
}

// The compile-time rule a plan can use (0: none).
inline int const_gp_points(int etype, int num_gp) {
  if (etype == FOLGB_QUAD4 && num_gp == 2) return 4;
  if (etype == FOLGB_TET4 && num_gp == 1) return 1;
  return 0;
}

template <int PH, int DIM> struct NdofT {
  static constexpr int V = (PH == FOLGB_THERMAL || PH == FOLGB_TRANSIENT_THERMAL) ? 1 : DIM;
};

// ---------------------------------------------------------------------------
// small dense helpers (fp32)
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ float det_inv(const float (&J)[D][D], float (&Ji)[D][D]);

template <>
__device__ __forceinline__ float det_inv<2>(const float (&J)[2][2], float (&Ji)[2][2]) {
  float det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  float r = 1.0f / det;
  Ji[0][0] = J[1][1] * r;
  Ji[0][1] = -J[0][1] * r;
  Ji[1][0] = -J[1][0] * r;
  Ji[1][1] = J[0][0] * r;
  return det;
}

template <>
__device__ __forceinline__ float det_inv<3>(const float (&J)[3][3], float (&Ji)[3][3]) {
  float c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  float c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  float c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  float det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  float r = 1.0f / det;
  Ji[0][0] = c00 * r;
  Ji[1][0] = c01 * r;
  Ji[2][0] = c02 * r;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
  return det;
}

// Saint-Venant-Kirchhoff material at one Gauss point
// (constitutive_material_models/saint_venant.py:13-31): E = (F^T F - I)/2,
// computed as (H + H^T + H^T H)/2 to keep small strains accurate in fp32,
// psi = lam/2 tr(E)^2 + mu E:E, S = lam tr(E) I + 2 mu E.  dpsi_de is the
// energy per unit Young's modulus (lam and mu are proportional to it).
template <int D>
struct SVKState {
  float F[D][D];
  float S[D][D];
  float psi, dpsi_de;
};

template <int D>
__device__ __forceinline__ void svk_state(const float (&H)[D][D], float mu, float lam, float mu1, float lam1,
                                          SVKState<D>& st) {
  float E[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      float hh = 0.f;
#pragma unroll
      for (int k = 0; k < D; ++k) hh = fmaf(H[k][i], H[k][j], hh);
      E[i][j] = 0.5f * (H[i][j] + H[j][i] + hh);
      st.F[i][j] = H[i][j] + (i == j ? 1.f : 0.f);
    }
  float tr = 0.f, ee = 0.f;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    tr += E[i][i];
#pragma unroll
    for (int j = 0; j < D; ++j) ee = fmaf(E[i][j], E[i][j], ee);
  }
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) st.S[i][j] = 2.f * mu * E[i][j] + (i == j ? lam * tr : 0.f);
  st.psi = 0.5f * lam * tr * tr + mu * ee;
  st.dpsi_de = 0.5f * lam1 * tr * tr + mu1 * ee;
}

// dS for a symmetric increment dC of C = F^T F (dE = dC / 2)
template <int D>
__device__ __forceinline__ void svk_dS(float mu, float lam, const float (&dC)[D][D], float (&dS)[D][D]) {
  float tr = 0.f;
#pragma unroll
  for (int i = 0; i < D; ++i) tr += 0.5f * dC[i][i];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) dS[i][j] = mu * dC[i][j] + (i == j ? lam * tr : 0.f);
}

// Neo-Hookean kinematics and stress at one Gauss point, written to avoid the
// fp32 cancellation of det(C) near C = I: J - 1 comes from the invariant
// expansion of det(I + H) and ln J from log1p.
//   psi = mu/2 (J^-2/3 I1 - 3) - mu lnJ + lam/2 ln^2 J           (3-D)
//   psi = mu/2 (I1 - 2)        - mu lnJ + lam/2 ln^2 J           (2-D)
// (fol/constitutive_material_models/neo_hooke.py:129-135, 178-181)
template <int D>
struct NHState {
  float F[D][D];
  float Ci[D][D];
  float S[D][D];   // true second Piola-Kirchhoff stress
  float lnJ, a, I1, psi, dpsi_dmu, dpsi_dlam;
};

template <int D>
__device__ __forceinline__ void nh_state(const float (&H)[D][D], float mu, float lam, NHState<D>& st) {
  float E[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < D; ++k) s = fmaf(H[k][i], H[k][j], s);
      E[i][j] = 0.5f * (H[i][j] + H[j][i] + s);
      st.F[i][j] = H[i][j] + (i == j ? 1.f : 0.f);
    }
  float trE = 0.f;
#pragma unroll
  for (int i = 0; i < D; ++i) trE += E[i][i];
  float Jm1;
  if constexpr (D == 3) {
    float m2 = H[0][0] * H[1][1] - H[0][1] * H[1][0] + H[0][0] * H[2][2] - H[0][2] * H[2][0] +
               H[1][1] * H[2][2] - H[1][2] * H[2][1];
    float dH = H[0][0] * (H[1][1] * H[2][2] - H[1][2] * H[2][1]) -
               H[0][1] * (H[1][0] * H[2][2] - H[1][2] * H[2][0]) +
               H[0][2] * (H[1][0] * H[2][1] - H[1][1] * H[2][0]);
    Jm1 = (H[0][0] + H[1][1] + H[2][2]) + m2 + dH;
  } else {
    Jm1 = (H[0][0] + H[1][1]) + (H[0][0] * H[1][1] - H[0][1] * H[1][0]);
  }
  float lnJ = log1pf(Jm1);
  float J = 1.f + Jm1;
  float detC = J * J;
  float C[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) C[i][j] = 2.f * E[i][j] + (i == j ? 1.f : 0.f);
  float rdet = 1.f / detC;
  if constexpr (D == 3) {
    st.Ci[0][0] = (C[1][1] * C[2][2] - C[1][2] * C[2][1]) * rdet;
    st.Ci[0][1] = (C[0][2] * C[2][1] - C[0][1] * C[2][2]) * rdet;
    st.Ci[0][2] = (C[0][1] * C[1][2] - C[0][2] * C[1][1]) * rdet;
    st.Ci[1][1] = (C[0][0] * C[2][2] - C[0][2] * C[2][0]) * rdet;
    st.Ci[1][2] = (C[0][2] * C[1][0] - C[0][0] * C[1][2]) * rdet;
    st.Ci[2][2] = (C[0][0] * C[1][1] - C[0][1] * C[1][0]) * rdet;
    st.Ci[1][0] = st.Ci[0][1];
    st.Ci[2][0] = st.Ci[0][2];
    st.Ci[2][1] = st.Ci[1][2];
    float I1 = 3.f + 2.f * trE;
    float am1 = expm1f(-2.f / 3.f * lnJ);
    float a = 1.f + am1;
    float iso = fmaf(am1, I1, 2.f * trE);  // J^-2/3 I1 - 3
    st.psi = 0.5f * mu * iso - mu * lnJ + 0.5f * lam * lnJ * lnJ;
    st.dpsi_dmu = 0.5f * iso - lnJ;
    st.dpsi_dlam = 0.5f * lnJ * lnJ;
    st.a = a;
    st.I1 = I1;
    float t = I1 * (1.f / 3.f);
    float cc = lam * lnJ - mu;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        st.S[i][j] = mu * a * ((i == j ? 1.f : 0.f) - t * st.Ci[i][j]) + cc * st.Ci[i][j];
  } else {
    st.Ci[0][0] = C[1][1] * rdet;
    st.Ci[1][1] = C[0][0] * rdet;
    st.Ci[0][1] = -C[0][1] * rdet;
    st.Ci[1][0] = st.Ci[0][1];
    float I1m2 = 2.f * trE;
    st.psi = 0.5f * mu * I1m2 - mu * lnJ + 0.5f * lam * lnJ * lnJ;
    st.dpsi_dmu = 0.5f * I1m2 - lnJ;
    st.dpsi_dlam = 0.5f * lnJ * lnJ;
    st.a = 1.f;
    st.I1 = 2.f + I1m2;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j)
        st.S[i][j] = mu * ((i == j ? 1.f : 0.f) - st.Ci[i][j]) + lam * lnJ * st.Ci[i][j];
  }
  st.lnJ = lnJ;
}

// The energy and its gradient P = dpsi/dF = F S of the same model without
// forming C, C^-1 or S: F C^-1 = F^-T = cof(F) / J, so
//   3-D: P = mu a F + ((lam lnJ - mu) - mu a I1 / 3) / J cof(F),  a = J^-2/3
//   2-D: P = mu F + (lam lnJ - mu) / J cof(F)
// (about 100 fewer operations per point than nh_state + F S).  J - 1, ln J and
// J^-2/3 I1 - 3 are formed from H as nh_state forms them, so small strains
// keep their digits.
template <int D>
__device__ __forceinline__ void nh_first_piola(const float (&H)[D][D], float mu, float lam, float (&P)[D][D],
                                               float& psi, float& dpsi_dmu, float& dpsi_dlam) {
  float F[D][D];
  float hh = 0.f, trH = 0.f;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    trH += H[i][i];
#pragma unroll
    for (int j = 0; j < D; ++j) {
      F[i][j] = H[i][j] + (i == j ? 1.f : 0.f);
      hh = fmaf(H[i][j], H[i][j], hh);
    }
  }
  const float trE = fmaf(0.5f, hh, trH);  // tr E, E = (H + H^T + H^T H) / 2
  float Jm1, cof[D][D];
  if constexpr (D == 3) {
    const float m2 = H[0][0] * H[1][1] - H[0][1] * H[1][0] + H[0][0] * H[2][2] - H[0][2] * H[2][0] +
                     H[1][1] * H[2][2] - H[1][2] * H[2][1];
    const float dH = H[0][0] * (H[1][1] * H[2][2] - H[1][2] * H[2][1]) -
                     H[0][1] * (H[1][0] * H[2][2] - H[1][2] * H[2][0]) +
                     H[0][2] * (H[1][0] * H[2][1] - H[1][1] * H[2][0]);
    Jm1 = trH + m2 + dH;
    cof[0][0] = F[1][1] * F[2][2] - F[1][2] * F[2][1];
    cof[0][1] = F[1][2] * F[2][0] - F[1][0] * F[2][2];
    cof[0][2] = F[1][0] * F[2][1] - F[1][1] * F[2][0];
    cof[1][0] = F[0][2] * F[2][1] - F[0][1] * F[2][2];
    cof[1][1] = F[0][0] * F[2][2] - F[0][2] * F[2][0];
    cof[1][2] = F[0][1] * F[2][0] - F[0][0] * F[2][1];
    cof[2][0] = F[0][1] * F[1][2] - F[0][2] * F[1][1];
    cof[2][1] = F[0][2] * F[1][0] - F[0][0] * F[1][2];
    cof[2][2] = F[0][0] * F[1][1] - F[0][1] * F[1][0];
  } else {
    Jm1 = trH + (H[0][0] * H[1][1] - H[0][1] * H[1][0]);
    cof[0][0] = F[1][1];
    cof[0][1] = -F[1][0];
    cof[1][0] = -F[0][1];
    cof[1][1] = F[0][0];
  }
  const float lnJ = log1pf(Jm1);
  const float rJ = 1.f / (1.f + Jm1);
  const float cc = lam * lnJ - mu;
  float ma, c2;
  if constexpr (D == 3) {
    const float I1 = fmaf(2.f, trE, 3.f);
    const float am1 = expm1f(-2.f / 3.f * lnJ);
    const float iso = fmaf(am1, I1, 2.f * trE);  // J^-2/3 I1 - 3
    psi = 0.5f * mu * iso - mu * lnJ + 0.5f * lam * lnJ * lnJ;
    dpsi_dmu = 0.5f * iso - lnJ;
    ma = mu * (1.f + am1);
    c2 = (cc - ma * I1 * (1.f / 3.f)) * rJ;
  } else {
    psi = mu * trE - mu * lnJ + 0.5f * lam * lnJ * lnJ;
    dpsi_dmu = trE - lnJ;
    ma = mu;
    c2 = cc * rJ;
  }
  dpsi_dlam = 0.5f * lnJ * lnJ;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) P[i][j] = fmaf(ma, F[i][j], c2 * cof[i][j]);
}

// Directional derivative dS of the true S along a symmetric dC.
template <int D>
__device__ __forceinline__ void nh_dS(const NHState<D>& st, float mu, float lam, const float (&dC)[D][D],
                                      float (&dS)[D][D]) {
  float CidC[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < D; ++k) s = fmaf(st.Ci[i][k], dC[k][j], s);
      CidC[i][j] = s;
    }
  float tr = 0.f;
#pragma unroll
  for (int i = 0; i < D; ++i) tr += CidC[i][i];
  float dCi[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < D; ++k) s = fmaf(CidC[i][k], st.Ci[k][j], s);
      dCi[i][j] = -s;
    }
  float dlnJ = 0.5f * tr;
  float cc = lam * st.lnJ - mu;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) dS[i][j] = lam * dlnJ * st.Ci[i][j] + cc * dCi[i][j];
  if constexpr (D == 3) {
    float da = -(1.f / 3.f) * st.a * tr;
    float dI1 = dC[0][0] + dC[1][1] + dC[2][2];
    float t = st.I1 * (1.f / 3.f);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        dS[i][j] += mu * (da * ((i == j ? 1.f : 0.f) - t * st.Ci[i][j]) -
                          st.a * (dI1 * (1.f / 3.f) * st.Ci[i][j] + t * dCi[i][j]));
  }
}

// x - log(1 + x) without the cancellation of the direct form near x = 0:
// x^2 sum_{k=2..11} (-1)^k x^(k-2) / k for |x| < 1/8 (truncation below
// 3e-9 relative), the direct form beyond (relative error ~ 2 eps / |x|).
__device__ __forceinline__ float x_minus_log1p(float x) {
  if (fabsf(x) < 0.125f) {
    float h = -1.f / 11.f;
#pragma unroll
    for (int k = 10; k >= 2; --k) h = fmaf(h, x, ((k & 1) ? -1.f : 1.f) / (float)k);
    return x * x * h;
  }
  return x - log1pf(x);
}

// exp(y) - 1 - y, the same way: y^2 sum_{k=2..11} y^(k-2) / k! for |y| < 1/8.
__device__ __forceinline__ float expm1_minus_x(float y) {
  if (fabsf(y) < 0.125f) {
    float h = 1.f / 39916800.f;  // 1/11!
    float f = 39916800.f;
#pragma unroll
    for (int k = 10; k >= 2; --k) {
      f /= (float)(k + 1);
      h = fmaf(h, y, 1.f / f);
    }
    return y * y * h;
  }
  return expm1f(y) - y;
}

// Neo-Hookean material with a volumetric-isochoric split at one Gauss point
// (fol/constitutive_material_models/neo_hooke.py:14-59 in 2-D, 64-111 in 3-D;
// used by fol/loss_functions/mechanical_neohooke.py:243-275), d = D:
//   psi = kappa/4 (J^2 - 2 lnJ - 1) + mu/2 (J^(-2/d) I1 - d)
//   S   = kappa/2 (J^2 - 1) C^-1 + mu J^(-2/d) (I - I1/d C^-1)
// The energy is second order in H = grad u, and the direct forms lose it to
// fp32 cancellation of first-order terms at small strains.  So, with
// J - 1 = tr H + m2(H) + det H (invariant expansion of det(I + H)) and
// tr E = tr H + |H|^2 / 2:
//   J^2 - 2 lnJ - 1       = (J-1)^2 + 2 ((J-1) - log1p(J-1))
//   J^(-2/d) I1 - d        = 2 (tr E - (J-1)) + 2 ((J-1) - log1p(J-1))
//                            + d (e^y - 1 - y) + 2 tr E (e^y - 1),  y = -2/d lnJ
//   I - I1/d C^-1          = 2 C^-1 dev(E)
// where tr E - (J-1) = |H|^2 / 2 - m2 - det H needs no first-order term.
// dpsi_dk and dpsi_dmu are the energy per unit kappa and mu.
template <int D>
struct NHSState {
  float F[D][D];
  float Ci[D][D];
  float S[D][D];
  float detCm1, a, I1, psi, dpsi_dk, dpsi_dmu;
};

template <int D>
__device__ __forceinline__ void nh_split_state(const float (&H)[D][D], float kappa, float mu, NHSState<D>& st) {
  float E[D][D];
  float hh = 0.f;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < D; ++k) s = fmaf(H[k][i], H[k][j], s);
      E[i][j] = 0.5f * (H[i][j] + H[j][i] + s);
      st.F[i][j] = H[i][j] + (i == j ? 1.f : 0.f);
      hh = fmaf(H[i][j], H[i][j], hh);
    }
  float trE = 0.f, trH = 0.f;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    trE += E[i][i];
    trH += H[i][i];
  }
  float q;  // tr E - (J - 1), second order
  if constexpr (D == 3) {
    const float m2 = H[0][0] * H[1][1] - H[0][1] * H[1][0] + H[0][0] * H[2][2] - H[0][2] * H[2][0] +
                     H[1][1] * H[2][2] - H[1][2] * H[2][1];
    const float dH = H[0][0] * (H[1][1] * H[2][2] - H[1][2] * H[2][1]) -
                     H[0][1] * (H[1][0] * H[2][2] - H[1][2] * H[2][0]) +
                     H[0][2] * (H[1][0] * H[2][1] - H[1][1] * H[2][0]);
    q = 0.5f * hh - m2 - dH;
    st.detCm1 = trH + m2 + dH;  // J - 1 for now
  } else {
    const float dH = H[0][0] * H[1][1] - H[0][1] * H[1][0];
    q = 0.5f * hh - dH;
    st.detCm1 = trH + dH;
  }
  const float Jm1 = st.detCm1;
  const float lnJ = log1pf(Jm1);
  const float J = 1.f + Jm1;
  const float rdet = 1.f / (J * J);
  float C[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) C[i][j] = 2.f * E[i][j] + (i == j ? 1.f : 0.f);
  if constexpr (D == 3) {
    st.Ci[0][0] = (C[1][1] * C[2][2] - C[1][2] * C[2][1]) * rdet;
    st.Ci[0][1] = (C[0][2] * C[2][1] - C[0][1] * C[2][2]) * rdet;
    st.Ci[0][2] = (C[0][1] * C[1][2] - C[0][2] * C[1][1]) * rdet;
    st.Ci[1][1] = (C[0][0] * C[2][2] - C[0][2] * C[2][0]) * rdet;
    st.Ci[1][2] = (C[0][2] * C[1][0] - C[0][0] * C[1][2]) * rdet;
    st.Ci[2][2] = (C[0][0] * C[1][1] - C[0][1] * C[1][0]) * rdet;
    st.Ci[1][0] = st.Ci[0][1];
    st.Ci[2][0] = st.Ci[0][2];
    st.Ci[2][1] = st.Ci[1][2];
  } else {
    st.Ci[0][0] = C[1][1] * rdet;
    st.Ci[1][1] = C[0][0] * rdet;
    st.Ci[0][1] = -C[0][1] * rdet;
    st.Ci[1][0] = st.Ci[0][1];
  }
  const float y = (-2.f / (float)D) * lnJ;
  const float am1 = expm1f(y);
  const float a = 1.f + am1;
  const float xl = x_minus_log1p(Jm1);
  const float iso = 2.f * q + 2.f * xl + (float)D * expm1_minus_x(y) + 2.f * trE * am1;  // J^(-2/d) I1 - d
  const float vol = fmaf(Jm1, Jm1, 2.f * xl);                                              // J^2 - 2 lnJ - 1
  st.detCm1 = Jm1 * (2.f + Jm1);                                                           // J^2 - 1
  st.dpsi_dk = 0.25f * vol;
  st.dpsi_dmu = 0.5f * iso;
  st.psi = kappa * st.dpsi_dk + mu * st.dpsi_dmu;
  st.a = a;
  st.I1 = (float)D + 2.f * trE;
  float dev[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) dev[i][j] = E[i][j] - (i == j ? trE * (1.f / (float)D) : 0.f);
  const float pv = 0.5f * kappa * st.detCm1;
  const float ma2 = 2.f * mu * a;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < D; ++k) s = fmaf(st.Ci[i][k], dev[k][j], s);
      st.S[i][j] = fmaf(pv, st.Ci[i][j], ma2 * s);
    }
}

// Directional derivative dS along a symmetric dC (half the reference's
// C_vol + C_iso tangent, neo_hooke.py:47-56, 99-108, applied to dC).
template <int D>
__device__ __forceinline__ void nh_split_dS(const NHSState<D>& st, float kappa, float mu, const float (&dC)[D][D],
                                            float (&dS)[D][D]) {
  float CidC[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < D; ++k) s = fmaf(st.Ci[i][k], dC[k][j], s);
      CidC[i][j] = s;
    }
  float tr = 0.f, dI1 = 0.f;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    tr += CidC[i][i];
    dI1 += dC[i][i];
  }
  float dCi[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < D; ++k) s = fmaf(CidC[i][k], st.Ci[k][j], s);
      dCi[i][j] = -s;
    }
  const float rd = 1.f / (float)D;
  const float ddet = (1.f + st.detCm1) * tr;
  const float da = -rd * st.a * tr;
  const float t = st.I1 * rd;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j)
      dS[i][j] = 0.5f * kappa * (ddet * st.Ci[i][j] + st.detCm1 * dCi[i][j]) +
                 mu * (da * ((i == j ? 1.f : 0.f) - t * st.Ci[i][j]) -
                       st.a * (dI1 * rd * st.Ci[i][j] + t * dCi[i][j]));
}

// Voigt index pairs: 3-D [xx,yy,zz,yz,xz,xy], 2-D [xx,yy,xy]
// (fol/constitutive_material_models/utils.py:13-32).
template <int D> struct Voigt;
template <> struct Voigt<3> {
  static constexpr int NV = 6;
  __device__ static constexpr int p(int v) { return v == 0 ? 0 : v == 1 ? 1 : v == 2 ? 2 : v == 3 ? 1 : 0; }
  __device__ static constexpr int q(int v) { return v == 0 ? 0 : v == 1 ? 1 : v == 2 ? 2 : v == 3 ? 2 : v == 4 ? 2 : 1; }
};
template <> struct Voigt<2> {
  static constexpr int NV = 3;
  __device__ static constexpr int p(int v) { return v == 0 ? 0 : v == 1 ? 1 : 0; }
  __device__ static constexpr int q(int v) { return v == 0 ? 0 : v == 1 ? 1 : 1; }
};

// deterministic block reduction of one float (blockDim multiple of 32, <= 1024)
__device__ __forceinline__ float block_sum(float v, float* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  int nw = blockDim.x >> 5;
  float r = 0.f;
  if (threadIdx.x < 32) {
    r = (l < nw) ? sh[l] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
  }
  return r;  // valid in thread 0
}

__device__ __forceinline__ double block_sum_d(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  int nw = blockDim.x >> 5;
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = (l < nw) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
  }
  return r;
}

}  // namespace folgb

namespace folgb {
// ---------------------------------------------------------------------------
// Opt-in kernel tracing: CUDA events recorded on the caller's stream around
// each kernel launch, summed per kernel id when read (folgb_trace_read).
// ---------------------------------------------------------------------------
enum KernelId {
  KID_ELEM_LOSS = 0,
  KID_GATHER = 1,
  KID_ELEM_MATRIX = 2,
  KID_PAIR_REDUCE = 3,
  KID_PLAIN_BACKWARD = 4,
  KID_ELEM_RESIDUAL = 5,
  KID_PCG_SPMV = 6,
  KID_PCG_UPDATE = 7,
  KID_BATCH_LOSS = 8,
  KID_HEX8_FUSED = 9,
  KID_COUNT = 16
};
void trace_begin(int kid, cudaStream_t s);
void trace_end(int kid, cudaStream_t s);
bool trace_active();

inline int loss_record(const folgb_plan* p) {
  return padded_record(p->ndof + (p->ctrl_layout == FOLGB_CONTROL_NODAL ? 1 : 0));
}
inline int residual_record(const folgb_plan* p) { return padded_record(p->ndof); }
}  // namespace folgb
