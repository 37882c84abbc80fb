// Element kernels: fused loss + adjoint, deterministic node gather, element
// matrices, CSR segmented reduction, and the plain (materialised Se) path.
//
// Reference behaviour restated here (paths inside the folax project):
//   gather by connectivity          fol/loss_functions/fe_loss.py:155-164, 232-248
//   isoparametric map               fol/geometries/geometry.py:87-97
//   thermal element                 fol/loss_functions/thermal.py:28-49
//   linear elastic element          fol/loss_functions/mechanical.py:98-117
//   Neo-Hookean (AD) element        fol/loss_functions/mechanical_neohooke_AD.py:254-293
//   batch loss                      fol/loss_functions/fe_loss.py:250-262
//   residual / Jacobian assembly    fol/loss_functions/fe_loss.py:191-207, 264-318
#include <cmath>
#include <type_traits>

#include "element_body.cuh"

using namespace folgb;

namespace folgb {

// One thread per element: gather, Gauss-point loop, element energy, element
// energy gradient (LOSS) or element residual (RESIDUAL).
// IFAST (batches): the grid is (instances, element blocks), so the blocks of
// all instances for one element range are dispatched together and share the
// connectivity and coordinate loads in L2 instead of each instance sweeping
// the whole mesh.  A block takes `tiles` consecutive ranges of blockDim.x
// elements (big batches: fewer, longer-lived blocks keep the SMs fuller than
// many short ones).  With a compile-time Gauss rule (NP > 0) the table in
// shared memory is not used and not loaded.
template <int ET, int PH, int MODE, bool IFAST = false, int NP = 0>
__global__ void __launch_bounds__(256) k_elem_vector(const VecArgs A, const int tiles) {
  __shared__ GPTable gp;
  __shared__ float wsum[32];
  __shared__ unsigned wcount;
  pdl_launch_dependents();
  if constexpr (NP == 0) load_gp_table(gp, A.gp);
  if (threadIdx.x == 0) wcount = 0u;
  __syncthreads();
  const int b = IFAST ? blockIdx.x : blockIdx.y;
  const int blk = IFAST ? blockIdx.y : blockIdx.x, nblk = IFAST ? gridDim.y : gridDim.x;
  float energy = 0.f;
  int bad = 0;
  for (int k = 0; k < tiles; ++k) {
    const int64_t e = ((int64_t)blk * tiles + k) * blockDim.x + threadIdx.x;
    if (e < A.E) elem_vector_body<ET, PH, MODE, NP>(A, gp, b, e, energy, bad);
  }
  // warp-level epilogues: no block barrier after the element work
  if constexpr (MODE == MODE_LOSS) finish_loss_warp(energy, bad, A, b, wsum, &wcount, blk, nblk);
  else report_bad_warp(bad, A.status);
}


struct GatherArgs {
  int64_t E, N;  // E: the record sources (elements, or tet patches)
  int nen;       // records per source
  int64_t E_ctrl;  // elements of the element-layout control gradient
  const int* inc_ptr;
  const int* inc_slot;
  const int* inc_padded;  // [N][pad] slots, -1 padded (pad 4 or 8), or NULL
  const unsigned char* dmask;
  const float* g;      // [B][nen][E] records of `rec` floats (local-node-major)
  int rec;             // record width: ndof, + 1 when it carries the control sensitivity
  int with_gde;        // record component ndof is the nodal control sensitivity
  const float* scale;  // [B] or NULL (scale 1)
  float* out;          // [B][ndof*N] or NULL
  int64_t out_stride;
  float* dctrl;        // [B][N] nodal control gradient or NULL
  int64_t dctrl_stride;
  float* dctrl_elem;   // [B][E] rescaled in place when rescale_elem != 0
  int rescale_elem;
  const int* node_inst;  // batched meshes: instance of each node (scale index), or NULL
  const int* elem_inst;  // batched meshes: instance of each element, or NULL
};

// Deterministic transpose-gather: node n sums the records of its incident
// (element, local node) slots in ascending element order (no float atomics).
// Every index and record load of a node is issued before the sums (vector
// loads: records are 4/8/16 bytes, and when no node has more than 4 or 8
// incidences the slot list is read from a -1 padded table with int4 loads),
// so a node costs two memory latencies, not one per slot.
// Dirichlet dofs get 0 (fe_loss.py:91-100 overwrites them, so their gradient
// is zero; the BC residual rows are zeroed by fe_loss.py:191-207).
template <int REC>
__device__ __forceinline__ void load_rec(const float* __restrict__ p, float (&v)[REC]) {
  if constexpr (REC == 4) {
    const float4 t = __ldg(reinterpret_cast<const float4*>(p));
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
    v[3] = t.w;
  } else if constexpr (REC == 2) {
    const float2 t = __ldg(reinterpret_cast<const float2*>(p));
    v[0] = t.x;
    v[1] = t.y;
  } else if constexpr (REC == 3) {  // unpadded 3-component records (tet patches)
    v[0] = __ldg(p);
    v[1] = __ldg(p + 1);
    v[2] = __ldg(p + 2);
  } else {
    v[0] = __ldg(p);
  }
}

template <int NDOF, int REC, bool GDE, int CH>
__device__ __forceinline__ void sum_slots(const float* __restrict__ g, const int (&slot)[CH], float (&acc)[NDOF],
                                          float& accd) {
  float v[CH][REC];
#pragma unroll
  for (int k = 0; k < CH; ++k) {
    if (slot[k] >= 0) load_rec<REC>(g + (int64_t)slot[k] * REC, v[k]);
    else {
#pragma unroll
      for (int c = 0; c < REC; ++c) v[k][c] = 0.f;
    }
  }
#pragma unroll
  for (int k = 0; k < CH; ++k) {
#pragma unroll
    for (int c = 0; c < NDOF; ++c) acc[c] += v[k][c];
    if constexpr (GDE) accd += v[k][NDOF];
  }
}

// PAD = 4 or 8: padded slot table; PAD = 0: CSR slot list in chunks of 8.
// IFAST (batches): grid (instances, node blocks), the instances of one node
// range dispatched together so they share the incidence loads in L2.
template <int NDOF, int REC, bool GDE, int PAD, bool IFAST = false>
__global__ void __launch_bounds__(256) k_node_gather(const GatherArgs A) {
  const int b = IFAST ? blockIdx.x : blockIdx.y;
  const int blk = IFAST ? blockIdx.y : blockIdx.x, nblk = IFAST ? gridDim.y : gridDim.x;
  const float* g = A.g + (int64_t)b * A.E * A.nen * REC;
  const int64_t stride = (int64_t)nblk * blockDim.x;
  float scb = 1.f;
  for (int64_t n = (int64_t)blk * blockDim.x + threadIdx.x; n < A.N; n += stride) {
    float acc[NDOF];
#pragma unroll
    for (int c = 0; c < NDOF; ++c) acc[c] = 0.f;
    float accd = 0.f;
    if constexpr (PAD > 0) {
      int slot[PAD];
      const int4* sp = reinterpret_cast<const int4*>(A.inc_padded + n * PAD);
#pragma unroll
      for (int k = 0; k < PAD / 4; ++k) {
        const int4 t = __ldg(sp + k);
        slot[4 * k] = t.x;
        slot[4 * k + 1] = t.y;
        slot[4 * k + 2] = t.z;
        slot[4 * k + 3] = t.w;
      }
      pdl_wait_primary();  // the incidence slots do not depend on the element kernel; the records do
      sum_slots<NDOF, REC, GDE, PAD>(g, slot, acc, accd);
    } else {
      constexpr int CH = 8;
      const int s0 = __ldg(A.inc_ptr + n), s1 = __ldg(A.inc_ptr + n + 1);
      pdl_wait_primary();
      for (int k0 = s0; k0 < s1; k0 += CH) {
        int slot[CH];
#pragma unroll
        for (int k = 0; k < CH; ++k) slot[k] = (k0 + k < s1) ? __ldg(A.inc_slot + k0 + k) : -1;
        sum_slots<NDOF, REC, GDE, CH>(g, slot, acc, accd);
      }
    }
    if (A.scale) scb = A.scale[b];
    const float sc = A.node_inst ? A.scale[__ldg(A.node_inst + n)] : scb;
    if (A.out) {
      const unsigned m = __ldg(A.dmask + n);
      float* o = A.out + (int64_t)b * A.out_stride + (int64_t)NDOF * n;
#pragma unroll
      for (int c = 0; c < NDOF; ++c) o[c] = ((m >> c) & 1u) ? 0.f : sc * acc[c];
    }
    if (A.dctrl) A.dctrl[(int64_t)b * A.dctrl_stride + n] = sc * accd;
  }
  if (A.rescale_elem && A.dctrl_elem) {
    pdl_wait_primary();
    if (A.scale) scb = A.scale[b];
    for (int64_t e = (int64_t)blk * blockDim.x + threadIdx.x; e < A.E_ctrl; e += stride)
      A.dctrl_elem[(int64_t)b * A.E_ctrl + e] *= A.elem_inst ? A.scale[__ldg(A.elem_inst + e)] : scb;
  }
}

// ---------------------------------------------------------------------------
// Element matrices.  Phase 1: one task per (element, Gauss point) writes the
// Gauss-point record (dN/dx, weights, and for neo-Hooke F, the used stress M
// and the Voigt tangent) to shared memory.  Phase 2: one task per
// (element, a, b) node-pair block sums its ndof x ndof block over the Gauss
// points, applies the transpose and the row-only Dirichlet rule, and stores it.
// ---------------------------------------------------------------------------
enum { MAT_ASSEMBLE = 0, MAT_PLAIN = 1 };

struct MatArgs {
  int64_t E;
  const int* conn;
  const float4* xyz4;
  const GPTable* gp;
  const float* ctrl;
  int64_t ctrl_stride;
  const float* dofs;
  int64_t dofs_stride;
  const unsigned char* dmask;
  const float* k0;
  const float* dval;
  int apply_dirichlet;
  int ctrl_layout;
  MatConst mat;
  int transpose;
  int epb;         // elements per block
  float* Ke;       // [B][E][nen][nen][ndof][ndof]
  float* Fe;       // plain: [B][E][nd] or NULL
  float* g;        // plain, nodal control: records (component ndof = control sensitivity)
  int rec;
  float* dctrl_elem;  // plain, element control: [B][E]
  float exponent, inv_batch;
  int* status;
};

template <int ET, int PH>
struct MatRec {
  static constexpr int NEN = ElemT<ET>::NEN, DIM = ElemT<ET>::DIM;
  static constexpr int NV = Voigt<DIM>::NV;
  static constexpr int GEO = NEN * DIM + 3;  // dNdx, wd, coef, sedw
  static constexpr int EXTRA = is_hyperelastic(PH) ? (2 * DIM * DIM + NV * NV)
                               : (PH == FOLGB_TRANSIENT_THERMAL ? NEN + 2 + DIM : 0);
  static constexpr int SIZE = GEO + EXTRA;
  static constexpr int O_WD = NEN * DIM, O_COEF = O_WD + 1, O_SED = O_WD + 2;
  static constexpr int O_F = GEO, O_M = GEO + DIM * DIM, O_HM = GEO + 2 * DIM * DIM;
  static constexpr int O_N = GEO, O_K = GEO + NEN, O_DK = GEO + NEN + 1, O_GT = GEO + NEN + 2;  // transient
};

template <int ET, int PH, int MMODE>
__global__ void __launch_bounds__(256) k_elem_matrix(const MatArgs A) {
  constexpr int NEN = ElemT<ET>::NEN, DIM = ElemT<ET>::DIM, NDOF = NdofT<PH, DIM>::V;
  constexpr int ND = NEN * NDOF;
  using R = MatRec<ET, PH>;
  constexpr int NV = R::NV;
  extern __shared__ float smem[];
  __shared__ GPTable gp;
  load_gp_table(gp, A.gp);
  __syncthreads();
  const int npts = gp.npts;
  const int b = blockIdx.y;
  const int64_t e0 = (int64_t)blockIdx.x * A.epb;
  const float* dofs = A.dofs ? A.dofs + (int64_t)b * A.dofs_stride : nullptr;
  const float* ctrl = A.ctrl + (int64_t)b * A.ctrl_stride;
  const MatConst& mt = A.mat;
  int bad = 0;
  // ---- phase 1
  for (int t = threadIdx.x; t < A.epb * npts; t += blockDim.x) {
    const int el = t / npts, q = t % npts;
    const int64_t e = e0 + el;
    if (e >= A.E) continue;
    float* rec = smem + (size_t)t * R::SIZE;
    int nodes[NEN];
    load_nodes<NEN>(A.conn, e, nodes);
    float X[NEN][3];
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
      float4 x = __ldg(A.xyz4 + nodes[a]);
      X[a][0] = x.x; X[a][1] = x.y; X[a][2] = x.z;
    }
    float J[DIM][DIM];
#pragma unroll
    for (int i = 0; i < DIM; ++i)
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        float s = 0.f;
#pragma unroll
        for (int a = 0; a < NEN; ++a) s = fmaf(X[a][i], dN_at<ET>(gp, q, a, k), s);
        J[i][k] = s;
      }
    float Ji[DIM][DIM];
    const float det = det_inv<DIM>(J, Ji);
    bad |= !(det > 0.f);
    const float wd = gp.w[q] * det;
    float dNdx[NEN][DIM];
#pragma unroll
    for (int a = 0; a < NEN; ++a)
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        float s = 0.f;
#pragma unroll
        // the transient thermal element uses J^-1 dN/dxi^T (transient_thermal.py:57-59)
        for (int k = 0; k < DIM; ++k)
          s = fmaf(dN_at<ET>(gp, q, a, k), PH == FOLGB_TRANSIENT_THERMAL ? Ji[j][k] : Ji[k][j], s);
        dNdx[a][j] = s;
        rec[a * DIM + j] = s;
      }
    float egp = 0.f;
    if (A.ctrl_layout == FOLGB_CONTROL_NODAL) {
#pragma unroll
      for (int a = 0; a < NEN; ++a) egp = fmaf(gp.N[q][a], __ldg(ctrl + nodes[a]), egp);
    } else {
      egp = __ldg(ctrl + e);
    }
    rec[R::O_WD] = wd;
    const bool need_u = is_hyperelastic(PH) || (PH == FOLGB_TRANSIENT_THERMAL) ||
                        (MMODE == MAT_PLAIN) ||
                        (PH == FOLGB_THERMAL && mt.beta != 0.f);
    float ue[ND];
    if (need_u) {
#pragma unroll
      for (int a = 0; a < NEN; ++a) {
        unsigned m = A.apply_dirichlet ? __ldg(A.dmask + nodes[a]) : 0u;
#pragma unroll
        for (int c = 0; c < NDOF; ++c) {
          int64_t d = (int64_t)NDOF * nodes[a] + c;
          ue[a * NDOF + c] = ((m >> c) & 1u) ? __ldg(A.dval + d) : __ldg(dofs + d);
        }
      }
    }
    if constexpr (PH == FOLGB_THERMAL) {
      float gf = 1.f, gg = 0.f;
      if (need_u) {
        float Tg = 0.f, gT[DIM] = {};
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
          Tg = fmaf(gp.N[q][a], ue[a], Tg);
#pragma unroll
          for (int j = 0; j < DIM; ++j) gT[j] = fmaf(ue[a], dNdx[a][j], gT[j]);
        }
        if (mt.beta != 0.f) gf = 1.f + mt.beta * powf(Tg, mt.c);
#pragma unroll
        for (int j = 0; j < DIM; ++j) gg = fmaf(gT[j], gT[j], gg);
      }
      rec[R::O_COEF] = wd * egp * gf;
      rec[R::O_SED] = wd * gf * gg;
    } else if constexpr (PH == FOLGB_ELASTIC) {
      rec[R::O_COEF] = wd * egp;
      float sed = 0.f;
      if (MMODE == MAT_PLAIN) {
        float H[DIM][DIM];
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
          for (int j = 0; j < DIM; ++j) {
            float s = 0.f;
#pragma unroll
            for (int a = 0; a < NEN; ++a) s = fmaf(ue[a * DIM + i], dNdx[a][j], s);
            H[i][j] = s;
          }
        float tr = 0.f, sq = 0.f, sh2 = 0.f;
#pragma unroll
        for (int i = 0; i < DIM; ++i) {
          tr += H[i][i];
          sq = fmaf(H[i][i], H[i][i], sq);
#pragma unroll
          for (int j = i + 1; j < DIM; ++j) sh2 = fmaf(H[i][j] + H[j][i], H[i][j] + H[j][i], sh2);
        }
        sed = mt.lam * tr * tr + 2.f * mt.mu * sq + mt.mu * sh2;
      }
      rec[R::O_SED] = wd * sed;
    } else if constexpr (PH == FOLGB_TRANSIENT_THERMAL) {
      float Tn = 0.f, kq = 0.f, gT[DIM];
#pragma unroll
      for (int j = 0; j < DIM; ++j) gT[j] = 0.f;
#pragma unroll
      for (int a = 0; a < NEN; ++a) {
        Tn = fmaf(gp.N[q][a], ue[a], Tn);
        kq = fmaf(gp.N[q][a], __ldg(A.k0 + nodes[a]), kq);
#pragma unroll
        for (int j = 0; j < DIM; ++j) gT[j] = fmaf(ue[a], dNdx[a][j], gT[j]);
        rec[R::O_N + a] = gp.N[q][a];
      }
      rec[R::O_COEF] = wd;
      rec[R::O_SED] = 0.f;
      rec[R::O_K] = kq * (1.f + mt.mbeta * powf(Tn, mt.c));
      rec[R::O_DK] = kq * mt.mbeta * mt.c * powf(Tn, mt.c - 1.f);
#pragma unroll
      for (int j = 0; j < DIM; ++j) rec[R::O_GT + j] = gT[j];
    } else if constexpr (PH == FOLGB_NEOHOOKE_SPLIT) {
      float H[DIM][DIM];
#pragma unroll
      for (int i = 0; i < DIM; ++i)
#pragma unroll
        for (int j = 0; j < DIM; ++j) {
          float s = 0.f;
#pragma unroll
          for (int a = 0; a < NEN; ++a) s = fmaf(ue[a * DIM + i], dNdx[a][j], s);
          H[i][j] = s;
        }
      const float kappa = mt.kap_f * egp, mu = mt.mu_f * egp;
      NHSState<DIM> st;
      nh_split_state<DIM>(H, kappa, mu, st);
      rec[R::O_COEF] = wd;
      rec[R::O_SED] = 0.f;
#pragma unroll
      for (int i = 0; i < DIM; ++i)
#pragma unroll
        for (int j = 0; j < DIM; ++j) {
          rec[R::O_F + i * DIM + j] = st.F[i][j];
          rec[R::O_M + i * DIM + j] = st.S[i][j];
        }
      // Voigt tangent dS_v / dC_w (the layout of the other hyperelastic models)
#pragma unroll
      for (int w = 0; w < NV; ++w) {
        float dC[DIM][DIM];
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
          for (int j = 0; j < DIM; ++j) dC[i][j] = 0.f;
        const int pw = Voigt<DIM>::p(w), qw = Voigt<DIM>::q(w);
        dC[pw][qw] = 1.f;
        dC[qw][pw] = 1.f;
        float dS[DIM][DIM];
        nh_split_dS<DIM>(st, kappa, mu, dC, dS);
#pragma unroll
        for (int v = 0; v < NV; ++v) rec[R::O_HM + v * NV + w] = dS[Voigt<DIM>::p(v)][Voigt<DIM>::q(v)];
      }
    } else if constexpr (PH == FOLGB_SAINT_VENANT) {
      float H[DIM][DIM];
#pragma unroll
      for (int i = 0; i < DIM; ++i)
#pragma unroll
        for (int j = 0; j < DIM; ++j) {
          float s = 0.f;
#pragma unroll
          for (int a = 0; a < NEN; ++a) s = fmaf(ue[a * DIM + i], dNdx[a][j], s);
          H[i][j] = s;
        }
      const float mu = mt.mu_f * egp, lam = mt.lam_f * egp;
      SVKState<DIM> st;
      svk_state<DIM>(H, mu, lam, mt.mu_f, mt.lam_f, st);
      rec[R::O_COEF] = wd;
      rec[R::O_SED] = 0.f;
#pragma unroll
      for (int i = 0; i < DIM; ++i)
#pragma unroll
        for (int j = 0; j < DIM; ++j) {
          rec[R::O_F + i * DIM + j] = st.F[i][j];
          rec[R::O_M + i * DIM + j] = st.S[i][j];
        }
      // Voigt tangent dS_v / dC_w (the same layout as the neo-Hookean one)
#pragma unroll
      for (int w = 0; w < NV; ++w) {
        float dC[DIM][DIM];
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
          for (int j = 0; j < DIM; ++j) dC[i][j] = 0.f;
        const int pw = Voigt<DIM>::p(w), qw = Voigt<DIM>::q(w);
        dC[pw][qw] = 1.f;
        dC[qw][pw] = 1.f;
        float dS[DIM][DIM];
        svk_dS<DIM>(mu, lam, dC, dS);
#pragma unroll
        for (int v = 0; v < NV; ++v) rec[R::O_HM + v * NV + w] = dS[Voigt<DIM>::p(v)][Voigt<DIM>::q(v)];
      }
    } else {
      float H[DIM][DIM];
#pragma unroll
      for (int i = 0; i < DIM; ++i)
#pragma unroll
        for (int j = 0; j < DIM; ++j) {
          float s = 0.f;
#pragma unroll
          for (int a = 0; a < NEN; ++a) s = fmaf(ue[a * DIM + i], dNdx[a][j], s);
          H[i][j] = s;
        }
      const float mu = mt.mu_f * egp, lam = mt.lam_f * egp;
      NHState<DIM> st;
      nh_state<DIM>(H, mu, lam, st);
      const float off = mt.shear_ref ? 2.f : 1.f;
      rec[R::O_COEF] = wd;
      rec[R::O_SED] = 0.f;
#pragma unroll
      for (int i = 0; i < DIM; ++i)
#pragma unroll
        for (int j = 0; j < DIM; ++j) {
          rec[R::O_F + i * DIM + j] = st.F[i][j];
          rec[R::O_M + i * DIM + j] = st.S[i][j] * (i == j ? 1.f : off);
        }
      // Voigt tangent of the used stress wrt the independent Voigt entries of C
#pragma unroll
      for (int w = 0; w < NV; ++w) {
        float dC[DIM][DIM];
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
          for (int j = 0; j < DIM; ++j) dC[i][j] = 0.f;
        const int pw = Voigt<DIM>::p(w), qw = Voigt<DIM>::q(w);
        dC[pw][qw] = 1.f;
        dC[qw][pw] = 1.f;
        float dS[DIM][DIM];
        nh_dS<DIM>(st, mu, lam, dC, dS);
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const int pv = Voigt<DIM>::p(v), qv = Voigt<DIM>::q(v);
          rec[R::O_HM + v * NV + w] = dS[pv][qv] * (pv == qv ? 1.f : off);
        }
      }
    }
  }
  __syncthreads();
  // ---- phase 2: node-pair blocks
  for (int t = threadIdx.x; t < A.epb * NEN * NEN; t += blockDim.x) {
    const int el = t / (NEN * NEN), ab = t % (NEN * NEN);
    const int a = ab / NEN, bb = ab % NEN;
    const int64_t e = e0 + el;
    if (e >= A.E) continue;
    // transposed assembly computes block (bb, a) and transposes it
    const int ra = (MMODE == MAT_ASSEMBLE && A.transpose) ? bb : a;
    const int rb = (MMODE == MAT_ASSEMBLE && A.transpose) ? a : bb;
    float K[NDOF][NDOF];
#pragma unroll
    for (int i = 0; i < NDOF; ++i)
#pragma unroll
      for (int j = 0; j < NDOF; ++j) K[i][j] = 0.f;
    for (int q = 0; q < npts; ++q) {
      const float* rec = smem + (size_t)(el * npts + q) * R::SIZE;
      float dNa[DIM], dNb[DIM];
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        dNa[j] = rec[ra * DIM + j];
        dNb[j] = rec[rb * DIM + j];
      }
      float dot = 0.f;
#pragma unroll
      for (int j = 0; j < DIM; ++j) dot = fmaf(dNa[j], dNb[j], dot);
      const float coef = rec[R::O_COEF];
      if constexpr (PH == FOLGB_THERMAL) {
        K[0][0] = fmaf(coef, dot, K[0][0]);
      } else if constexpr (PH == FOLGB_TRANSIENT_THERMAL) {
        // Me + dt (dK/dT N_a (grad T . grad N_b) + K grad N_a . grad N_b), as
        // transient_thermal.py:64-76 writes it
        float gTb = 0.f;
#pragma unroll
        for (int j = 0; j < DIM; ++j) gTb = fmaf(rec[R::O_GT + j], dNb[j], gTb);
        const float Na = rec[R::O_N + ra], Nb = rec[R::O_N + rb];
        const float v = mt.rho_cp * Na * Nb + mt.dt * (rec[R::O_DK] * Na * gTb + rec[R::O_K] * dot);
        K[0][0] = fmaf(coef, v, K[0][0]);
      } else if constexpr (PH == FOLGB_ELASTIC) {
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
          for (int j = 0; j < DIM; ++j) {
            float v = mt.lam * dNa[i] * dNb[j] + mt.mu * dNa[j] * dNb[i] + (i == j ? mt.mu * dot : 0.f);
            K[i][j] = fmaf(coef, v, K[i][j]);
          }
      } else {
        float F[DIM][DIM], M[DIM][DIM];
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
          for (int j = 0; j < DIM; ++j) {
            F[i][j] = rec[R::O_F + i * DIM + j];
            M[i][j] = rec[R::O_M + i * DIM + j];
          }
        // B_v(a,i) and Bc_w(b,l) = d c_w / d u_(b,l)
        float Ba[DIM][NV], Bc[DIM][NV];
#pragma unroll
        for (int k = 0; k < DIM; ++k)
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            const int p = Voigt<DIM>::p(v), qq = Voigt<DIM>::q(v);
            if (p == qq) {
              Ba[k][v] = F[k][p] * dNa[p];
              Bc[k][v] = 2.f * F[k][p] * dNb[p];
            } else {
              Ba[k][v] = F[k][p] * dNa[qq] + F[k][qq] * dNa[p];
              Bc[k][v] = F[k][p] * dNb[qq] + F[k][qq] * dNb[p];
            }
          }
#pragma unroll
        for (int l = 0; l < DIM; ++l) {
          float Z[NV];
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            float s = 0.f;
#pragma unroll
            for (int w = 0; w < NV; ++w) s = fmaf(rec[R::O_HM + v * NV + w], Bc[l][w], s);
            Z[v] = s;
          }
#pragma unroll
          for (int i = 0; i < DIM; ++i) {
            float s = 0.f;
#pragma unroll
            for (int v = 0; v < NV; ++v) s = fmaf(Ba[i][v], Z[v], s);
            K[i][l] = fmaf(coef, s, K[i][l]);
          }
        }
        float geo = 0.f;
#pragma unroll
        for (int p = 0; p < DIM; ++p)
#pragma unroll
          for (int qq = 0; qq < DIM; ++qq) geo = fmaf(dNa[p] * M[p][qq], dNb[qq], geo);
#pragma unroll
        for (int i = 0; i < DIM; ++i) K[i][i] = fmaf(coef, geo, K[i][i]);
      }
    }
    float out[NDOF][NDOF];
#pragma unroll
    for (int i = 0; i < NDOF; ++i)
#pragma unroll
      for (int j = 0; j < NDOF; ++j)
        out[i][j] = (MMODE == MAT_ASSEMBLE && A.transpose) ? K[j][i] : K[i][j];
    if (MMODE == MAT_ASSEMBLE) {
      // row-only Dirichlet (fe_loss.py:191-207): zero row (a,i), keep its diagonal
      const int na = __ldg(A.conn + e * NEN + a);
      const unsigned m = __ldg(A.dmask + na);
#pragma unroll
      for (int i = 0; i < NDOF; ++i)
        if ((m >> i) & 1u) {
#pragma unroll
          for (int j = 0; j < NDOF; ++j)
            if (!(a == bb && i == j)) out[i][j] = 0.f;
        }
    }
    float* dst = A.Ke + ((((int64_t)b * A.E + e) * NEN + a) * NEN + bb) * (NDOF * NDOF);
#pragma unroll
    for (int i = 0; i < NDOF; ++i)
#pragma unroll
      for (int j = 0; j < NDOF; ++j) dst[i * NDOF + j] = out[i][j];
  }
  if (MMODE == MAT_PLAIN) {
    // per (element, node): control sensitivity and body-force vector
    for (int t = threadIdx.x; t < A.epb * NEN; t += blockDim.x) {
      const int el = t / NEN, a = t % NEN;
      const int64_t e = e0 + el;
      if (e >= A.E) continue;
      float gd = 0.f, fw = 0.f;
      for (int q = 0; q < npts; ++q) {
        const float* rec = smem + (size_t)(el * npts + q) * R::SIZE;
        gd = fmaf(rec[R::O_SED], gp.N[q][a], gd);
        fw = fmaf(rec[R::O_WD], gp.N[q][a], fw);
      }
      if (A.ctrl_layout == FOLGB_CONTROL_NODAL)
        A.g[(((int64_t)b * NEN + a) * A.E + e) * A.rec + NDOF] = gd;
      if (A.Fe) {
#pragma unroll
        for (int i = 0; i < NDOF; ++i)
          A.Fe[(((int64_t)b * A.E + e) * NEN + a) * NDOF + i] = (PH == FOLGB_THERMAL) ? 0.f : fw * mt.bf[i];
      }
    }
    if (A.ctrl_layout != FOLGB_CONTROL_NODAL && A.dctrl_elem) {
      for (int el = threadIdx.x; el < A.epb; el += blockDim.x) {
        const int64_t e = e0 + el;
        if (e >= A.E) continue;
        float s = 0.f;
        for (int q = 0; q < npts; ++q) {
          const float* rec = smem + (size_t)(el * npts + q) * R::SIZE;
          float nsum = 0.f;
          for (int a = 0; a < NEN; ++a) nsum += gp.N[q][a];
          s = fmaf(rec[R::O_SED], nsum, s);
        }
        A.dctrl_elem[(int64_t)b * A.E + e] = (A.exponent == 1.f) ? s * A.inv_batch : s;
      }
    }
  }
  int anybad = __syncthreads_or(bad);
  if (anybad && threadIdx.x == 0 && A.status) atomicOr(A.status, 1 << FOLGB_ERR_NONPOSITIVE_DETJ);
}

// Segmented reduction over the element-to-nonzero map: one thread per node
// pair sums its contributing element blocks in ascending element order and
// writes the ndof x ndof block into the canonical CSR rows.
template <int NDOF>
__global__ void __launch_bounds__(256) k_pair_reduce(int64_t P, const int* __restrict__ pair_row,
                                                     const int* __restrict__ adj_ptr, const int* __restrict__ adj,
                                                     const int* __restrict__ pair_ptr, const int* __restrict__ pair_slot,
                                                     const int* __restrict__ rowptr, const float* __restrict__ Ke,
                                                     float* __restrict__ vals, float* __restrict__ inv_diag) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += stride) {
    const int n = __ldg(pair_row + p);
    const int j = (int)(p - __ldg(adj_ptr + n));
    const int m = __ldg(adj + p);
    float acc[NDOF * NDOF];
#pragma unroll
    for (int i = 0; i < NDOF * NDOF; ++i) acc[i] = 0.f;
    const int k0 = __ldg(pair_ptr + p), k1 = __ldg(pair_ptr + p + 1);
    for (int k = k0; k < k1; ++k) {
      const float* blk = Ke + (int64_t)__ldg(pair_slot + k) * (NDOF * NDOF);
#pragma unroll
      for (int i = 0; i < NDOF * NDOF; ++i) acc[i] += __ldg(blk + i);
    }
    if (vals) {
#pragma unroll
      for (int i = 0; i < NDOF; ++i) {
        float* row = vals + __ldg(rowptr + (int64_t)NDOF * n + i) + NDOF * j;
#pragma unroll
        for (int l = 0; l < NDOF; ++l) row[l] = acc[i * NDOF + l];
      }
    }
    if (inv_diag && m == n) {
#pragma unroll
      for (int i = 0; i < NDOF; ++i) inv_diag[(int64_t)NDOF * n + i] = 1.f / acc[i * NDOF + i];
    }
  }
}

// Plain backward pass: re = Se ue - Fe from the materialised element matrix,
// energy = ue . re, loss reduction (thermal / linear elastic only).
template <int ET, int PH>
__global__ void __launch_bounds__(256) k_plain_backward(const VecArgs A, const float* __restrict__ Ke,
                                                        const float* __restrict__ Fe) {
  constexpr int NEN = ElemT<ET>::NEN, DIM = ElemT<ET>::DIM, NDOF = NdofT<PH, DIM>::V;
  constexpr int ND = NEN * NDOF;
  __shared__ float red[32];
  const int b = blockIdx.y;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float energy = 0.f;
  if (e < A.E) {
    int nodes[NEN];
    load_nodes<NEN>(A.conn, e, nodes);
    const float* dofs = A.dofs + (int64_t)b * A.dofs_stride;
    float ue[ND];
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
      unsigned m = A.apply_dirichlet ? __ldg(A.dmask + nodes[a]) : 0u;
#pragma unroll
      for (int c = 0; c < NDOF; ++c) {
        int64_t d = (int64_t)NDOF * nodes[a] + c;
        ue[a * NDOF + c] = ((m >> c) & 1u) ? __ldg(A.dval + d) : __ldg(dofs + d);
      }
    }
    float r[ND];
#pragma unroll
    for (int i = 0; i < ND; ++i) r[i] = 0.f;
    const float4* K4 = reinterpret_cast<const float4*>(Ke + ((int64_t)b * A.E + e) * ND * ND);
    // element matrix layout [a][b][i][j]; flat index f -> (a,b,i,j)
#pragma unroll
    for (int f4 = 0; f4 < ND * ND / 4; ++f4) {
      float4 v = __ldg(K4 + f4);
      float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        const int f = 4 * f4 + s;
        const int blk = f / (NDOF * NDOF), ij = f % (NDOF * NDOF);
        const int a = blk / NEN, bb = blk % NEN, i = ij / NDOF, j = ij % NDOF;
        r[a * NDOF + i] = fmaf(vv[s], ue[bb * NDOF + j], r[a * NDOF + i]);
      }
    }
    if (Fe) {
#pragma unroll
      for (int i = 0; i < ND; ++i) r[i] -= __ldg(Fe + ((int64_t)b * A.E + e) * ND + i);
    }
#pragma unroll
    for (int i = 0; i < ND; ++i) energy = fmaf(ue[i], r[i], energy);
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
      float* rec = A.g + (((int64_t)b * NEN + a) * A.E + e) * A.rec;
#pragma unroll
      for (int c = 0; c < NDOF; ++c) rec[c] = r[a * NDOF + c];
    }
  }
  float be = block_sum(energy, red);
  finish_loss(be, A, b, red);
}

// ---------------------------------------------------------------------------
// workspace layouts
// ---------------------------------------------------------------------------
struct LossWS {
  float* g;
  int rec;
  float* partials;
  unsigned* counters;
  float* scale;
  float* Ke;
  float* Fe;
};

static int loss_blocks(const folgb_plan* p) { return (int)((p->E + 255) / 256); }
// element ranges per block of k_elem_vector: up to 16 while the launch keeps
// at least 8 waves of 4 blocks per SM (tet4 neo-Hooke, 64^3 split x 16: 1, 2,
// 4, 8, 16 ranges gave 1.11, 1.01, 0.93, 0.91, 0.90 ms per step)
static int elem_tiles(int64_t nb, int B) {
  int t = 1;
  while (t < 16 && ((nb + 2 * t - 1) / (2 * t)) * B >= (int64_t)32 * num_sms()) t *= 2;
  return t;
}
// partial-sum slots: enough for the smallest element-kernel block (64 threads)
// and for one per tile of the tile-local kernel
static int loss_partial_slots(const folgb_plan* p) {
  int64_t slots = (p->E + 63) / 64;
  if (p->tiles > slots) slots = p->tiles;
  if (p->box_grid) slots = std::max<int64_t>(slots, grid_blocks_max(p));
  return (int)slots;
}

// record width of the loss path: ndof components (+ the nodal control sensitivity)
static int loss_rec(const folgb_plan* p) { return loss_record(p); }

static size_t layout_loss(const folgb_plan* p, int B, bool plain, void* base, size_t cap, LossWS* w) {
  Bump bp(base, cap);
  const int64_t ND = (int64_t)p->nen * p->ndof;
  const int rec = loss_rec(p);
  // element records of the node gather, or the boundary partial records of
  // the tile-local kernel (4 floats per slot): the same region serves both
  const size_t recs = (size_t)B * p->E * p->nen * rec, parts = (size_t)B * p->tile_boundary_slots * 4;
  float* g = bp.take<float>(recs > parts ? recs : parts);
  float* partials = bp.take<float>((size_t)B * loss_partial_slots(p));
  unsigned* counters = bp.take<unsigned>((size_t)2 * B);  // [B] last-block counters, [B] tile queues
  float* scale = bp.take<float>((size_t)B);
  float* Ke = plain ? bp.take<float>((size_t)B * p->E * ND * ND) : nullptr;
  float* Fe = (plain && p->mat.has_bf) ? bp.take<float>((size_t)B * p->E * ND) : nullptr;
  if (w) *w = LossWS{g, rec, partials, counters, scale, Ke, Fe};
  return align_up(bp.off);
}

static size_t layout_assemble(const folgb_plan* p, void* base, size_t cap, float** g, float** Ke) {
  Bump bp(base, cap);
  const int64_t ND = (int64_t)p->nen * p->ndof;
  float* gg = bp.take<float>((size_t)p->E * p->nen * residual_record(p));
  float* kk = bp.take<float>((size_t)p->E * ND * ND);
  if (g) *g = gg;
  if (Ke) *Ke = kk;
  return align_up(bp.off);
}

size_t pcg_workspace_bytes(const folgb_plan* p);
size_t krylov64_workspace_bytes(const folgb_plan* p);

static int mat_epb(int rec_size, int npts) {
  const int budget = 96 * 1024;
  int epb = budget / (rec_size * npts * 4);
  if (epb > 32) epb = 32;
  if (epb < 1) epb = 1;
  return epb;
}

template <int ET, int PH, int MMODE>
static int launch_matrix(const MatArgs& A0, int B, int npts, cudaStream_t s) {
  using R = MatRec<ET, PH>;
  MatArgs A = A0;
  A.epb = mat_epb(R::SIZE, npts);
  const size_t shm = (size_t)A.epb * npts * R::SIZE * sizeof(float);
  FOLGB_CUDA_TRY(cudaFuncSetAttribute(k_elem_matrix<ET, PH, MMODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)shm));
  dim3 grid((unsigned)((A.E + A.epb - 1) / A.epb), (unsigned)B);
  trace_begin(KID_ELEM_MATRIX, s);
  k_elem_matrix<ET, PH, MMODE><<<grid, 256, shm, s>>>(A);
  trace_end(KID_ELEM_MATRIX, s);
  FOLGB_LAUNCH_CHECK();
  return FOLGB_OK;
}

int launch_gather(const folgb_plan* p, int B, const float* g, int rec, int with_gde, const float* scale, float* out,
                  int64_t out_stride, float* dctrl, int64_t dctrl_stride, float* dctrl_elem, int rescale_elem,
                  cudaStream_t s, const int* node_inst, const int* elem_inst, int pdl, int patches) {
  GatherArgs G;
  G.node_inst = node_inst;
  G.elem_inst = elem_inst;
  G.E = patches ? p->n_patches : p->E;
  G.N = p->N;
  G.nen = patches ? kPatchNodes : p->nen;
  G.E_ctrl = p->E;
  G.inc_ptr = patches ? p->d_patch_inc_ptr : p->d_inc_ptr;
  G.inc_slot = patches ? p->d_patch_inc_slot : p->d_inc_slot;
  G.inc_padded = patches ? p->d_patch_inc_padded : p->d_inc_padded;
  const int inc_pad = patches ? p->patch_pad : p->inc_pad;
  G.dmask = p->d_dmask;
  G.g = g;
  G.rec = rec;
  G.with_gde = with_gde;
  G.scale = scale;
  G.out = out;
  G.out_stride = out_stride;
  G.dctrl = dctrl;
  G.dctrl_stride = dctrl_stride;
  G.dctrl_elem = dctrl_elem;
  G.rescale_elem = rescale_elem;
  // unpadded 12-byte records: the tet patch kernel with element controls
  const bool rec3 = patches && rec == 3 && p->ndof == 3 && !with_gde;
  if (rec != padded_record(p->ndof + (with_gde ? 1 : 0)) && !rec3) return FOLGB_ERR_INVALID_ARGUMENT;
  int64_t work = p->N > p->E ? p->N : p->E;
  int blocks = (int)((work + 255) / 256);
  int cap = num_sms() * 8;
  if (blocks > cap) blocks = cap;
  const bool ifast = B > 1;  // blocks <= num_sms * 8 < 65536
  dim3 grid = ifast ? dim3((unsigned)B, (unsigned)blocks) : dim3((unsigned)blocks, (unsigned)B);
  auto go = [&](auto nd, auto rc_, auto gde) -> int {
    constexpr int NDOF = decltype(nd)::value, REC = decltype(rc_)::value;
    constexpr bool GDE = decltype(gde)::value;
    auto kernel = inc_pad == 4 ? (ifast ? k_node_gather<NDOF, REC, GDE, 4, true> : k_node_gather<NDOF, REC, GDE, 4>)
                  : (inc_pad == 8 ? (ifast ? k_node_gather<NDOF, REC, GDE, 8, true> : k_node_gather<NDOF, REC, GDE, 8>)
                                     : (ifast ? k_node_gather<NDOF, REC, GDE, 0, true> : k_node_gather<NDOF, REC, GDE, 0>));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    FOLGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, kernel, G));
    return (int)FOLGB_OK;
  };
  using I1 = std::integral_constant<int, 1>;
  using I2 = std::integral_constant<int, 2>;
  using I3 = std::integral_constant<int, 3>;
  using I4 = std::integral_constant<int, 4>;
  using T = std::true_type;
  using F = std::false_type;
  trace_begin(KID_GATHER, s);
  int rcode;
  switch (p->ndof * 2 + (with_gde ? 1 : 0)) {
    case 2: rcode = go(I1{}, I1{}, F{}); break;
    case 3: rcode = go(I1{}, I2{}, T{}); break;
    case 4: rcode = go(I2{}, I2{}, F{}); break;
    case 5: rcode = go(I2{}, I4{}, T{}); break;
    case 6: rcode = rec3 ? go(I3{}, std::integral_constant<int, 3>{}, F{}) : go(I3{}, I4{}, F{}); break;
    case 7: rcode = go(I3{}, I4{}, T{}); break;
    default: return FOLGB_ERR_INVALID_ARGUMENT;
  }
  trace_end(KID_GATHER, s);
  if (rcode) return rcode;
  FOLGB_LAUNCH_CHECK();
  return FOLGB_OK;
}

static VecArgs make_vec_args(const folgb_plan* p, int B, const float* control, int64_t cstride, const float* dofs,
                             int64_t dstride, int apply_dirichlet, const LossWS& w, float* losses,
                             float* dctrl_elem, int* status) {
  VecArgs A;
  A.E = p->E;
  A.N = p->N;
  A.conn = p->d_conn;
  A.xyz4 = p->d_xyz4;
  A.gp = p->d_gp;
  A.ctrl = control;
  A.ctrl_stride = cstride;
  A.dofs = dofs;
  A.dofs_stride = dstride;
  A.dmask = p->d_dmask;
  A.elem_bc = p->d_elem_bc;
  A.k0 = p->d_k0;
  A.dval = p->d_dval;
  A.apply_dirichlet = apply_dirichlet;
  A.ctrl_layout = p->ctrl_layout;
  A.mat = p->mat;
  A.g = w.g;
  A.rec = w.rec;
  A.dctrl_elem = dctrl_elem;
  A.partials = w.partials;
  A.counters = w.counters;
  A.losses = losses;
  A.scale = w.scale;
  A.exponent = (float)p->phys.loss_exponent;
  A.inv_batch = 1.f / (float)B;
  A.status = status;
  // records far larger than L2 are written evict-first (they are read back
  // from HBM by the gather in any case)
  A.stream_rec = (size_t)B * p->E * p->nen * w.rec * sizeof(float) > ((size_t)96 << 20) ? 1 : 0;
  return A;
}

static int check_loss_args(const folgb_plan* p, int B, const float* control, const float* dofs, const float* losses) {
  if (!p || B <= 0 || !control || !dofs || !losses) return FOLGB_ERR_INVALID_ARGUMENT;
  if (B > 65535) return FOLGB_ERR_INVALID_ARGUMENT;
  return FOLGB_OK;
}

}  // namespace folgb

using namespace folgb;

extern "C" size_t folgb_workspace_bytes(const folgb_plan* p, int32_t op, int32_t batch) {
  if (!p || batch <= 0) return 0;
  switch (op) {
    case FOLGB_OP_LOSS_ADJOINT: return layout_loss(p, batch, false, nullptr, 0, nullptr);
    case FOLGB_OP_PLAIN: return layout_loss(p, batch, true, nullptr, 0, nullptr);
    case FOLGB_OP_ASSEMBLE: return layout_assemble(p, nullptr, 0, nullptr, nullptr);
    case FOLGB_OP_PCG: return pcg_workspace_bytes(p);
    case FOLGB_OP_KRYLOV64: return krylov64_workspace_bytes(p);
  }
  return 0;
}

extern "C" int folgb_loss_adjoint(const folgb_plan* p, int32_t B, const float* control, int64_t control_stride,
                                  const float* dofs, int64_t dofs_stride, int32_t apply_dirichlet, float* losses,
                                  float* dloss_ddofs, float* dloss_dcontrol, int32_t* device_status, void* workspace,
                                  size_t workspace_bytes, void* stream) {
  int rc = check_loss_args(p, B, control, dofs, losses);
  if (rc) return rc;
  LossWS w;
  size_t need = layout_loss(p, B, false, workspace, workspace_bytes, &w);
  if (!workspace || workspace_bytes < need) return FOLGB_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  FOLGB_CUDA_TRY(cudaMemsetAsync(w.counters, 0, sizeof(unsigned) * 2 * B, s));
  const bool elem_ctrl = p->ctrl_layout == FOLGB_CONTROL_ELEMENT;
  VecArgs A = make_vec_args(p, B, control, control_stride, dofs, dofs_stride, apply_dirichlet, w, losses,
                            elem_ctrl ? dloss_dcontrol : nullptr, device_status);
  A.out = dloss_ddofs;
  A.out_stride = (int64_t)p->ndof * p->N;
  A.dctrl_nodal = elem_ctrl ? nullptr : dloss_dcontrol;
  dim3 grid((unsigned)loss_blocks(p), (unsigned)B);
  const int fast = p->phys.kernel_variant != 1 ? launch_hex8_fast(p, A, grid, MODE_LOSS, s) : 0;
  // tetrahedra in patches of six: one record per patch node
  const int patched = fast ? 0 : launch_tet_patch(p, A, B, s);
  if (patched < 0) return -patched;
  if (fast || patched) {
    FOLGB_LAUNCH_CHECK();
  } else {
    rc = dispatch(p->etype, p->physics, [&](auto tag) -> int {
      constexpr int ET = decltype(tag)::ET, PH = decltype(tag)::PH;
      trace_begin(KID_ELEM_LOSS, s);
      with_const_gp<ET>(p, [&](auto np) {
        constexpr int NP = decltype(np)::value;
        const int tiles = elem_tiles(grid.x, (int)grid.y);
        const unsigned nb = (unsigned)((grid.x + tiles - 1) / tiles);
        if (grid.y > 1 && nb <= 65535u)
          k_elem_vector<ET, PH, MODE_LOSS, true, NP><<<dim3(grid.y, nb), 256, 0, s>>>(A, tiles);
        else
          k_elem_vector<ET, PH, MODE_LOSS, false, NP><<<dim3(nb, grid.y), 256, 0, s>>>(A, tiles);
      });
      trace_end(KID_ELEM_LOSS, s);
      FOLGB_LAUNCH_CHECK();
      return FOLGB_OK;
    });
  }
  if (rc) return rc;
  if (fast == 3) {
    // the structured box grid kernel wrote the gradients itself
  } else if (fast == 2 && (dloss_ddofs || dloss_dcontrol)) {
    rc = launch_tile_boundary(p, A, B, s, trace_active() ? 0 : 1);
  } else if (dloss_ddofs || dloss_dcontrol) {
    rc = launch_gather(p, B, w.g, patched ? tet_patch_record(p) : w.rec, elem_ctrl ? 0 : 1, w.scale, dloss_ddofs,
                       (int64_t)p->ndof * p->N, elem_ctrl ? nullptr : dloss_dcontrol, p->N,
                       elem_ctrl ? dloss_dcontrol : nullptr, (elem_ctrl && p->phys.loss_exponent != 1.0) ? 1 : 0, s,
                       nullptr, nullptr, trace_active() ? 0 : 1, patched ? 1 : 0);
  }
  return rc;
}

extern "C" int folgb_loss_adjoint_plain(const folgb_plan* p, int32_t B, const float* control, int64_t control_stride,
                                        const float* dofs, int64_t dofs_stride, int32_t apply_dirichlet,
                                        float* losses, float* dloss_ddofs, float* dloss_dcontrol,
                                        int32_t* device_status, void* workspace, size_t workspace_bytes,
                                        void* stream) {
  int rc = check_loss_args(p, B, control, dofs, losses);
  if (rc) return rc;
  if (is_hyperelastic(p->physics) || p->physics == FOLGB_TRANSIENT_THERMAL) return FOLGB_ERR_INVALID_ARGUMENT;
  LossWS w;
  size_t need = layout_loss(p, B, true, workspace, workspace_bytes, &w);
  if (!workspace || workspace_bytes < need) return FOLGB_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  FOLGB_CUDA_TRY(cudaMemsetAsync(w.counters, 0, sizeof(unsigned) * 2 * B, s));
  const bool elem_ctrl = p->ctrl_layout == FOLGB_CONTROL_ELEMENT;
  MatArgs M;
  M.E = p->E;
  M.conn = p->d_conn;
  M.xyz4 = p->d_xyz4;
  M.gp = p->d_gp;
  M.ctrl = control;
  M.ctrl_stride = control_stride;
  M.dofs = dofs;
  M.dofs_stride = dofs_stride;
  M.dmask = p->d_dmask;
  M.k0 = p->d_k0;
  M.dval = p->d_dval;
  M.apply_dirichlet = apply_dirichlet;
  M.ctrl_layout = p->ctrl_layout;
  M.mat = p->mat;
  M.transpose = 0;
  M.epb = 0;
  M.Ke = w.Ke;
  M.Fe = w.Fe;
  M.g = w.g;
  M.rec = w.rec;
  M.dctrl_elem = elem_ctrl ? dloss_dcontrol : nullptr;
  M.exponent = (float)p->phys.loss_exponent;
  M.inv_batch = 1.f / (float)B;
  M.status = device_status;
  VecArgs A = make_vec_args(p, B, control, control_stride, dofs, dofs_stride, apply_dirichlet, w, losses,
                            elem_ctrl ? dloss_dcontrol : nullptr, device_status);
  const int npts = p->h_gp.npts;
  dim3 grid((unsigned)loss_blocks(p), (unsigned)B);
  rc = dispatch(p->etype, p->physics, [&](auto tag) -> int {
    constexpr int ET = decltype(tag)::ET, PH = decltype(tag)::PH;
    if constexpr (is_hyperelastic(PH) || PH == FOLGB_TRANSIENT_THERMAL) {
      return (int)FOLGB_ERR_INVALID_ARGUMENT;
    } else {
      int r = launch_matrix<ET, PH, MAT_PLAIN>(M, B, npts, s);
      if (r) return r;
      trace_begin(KID_PLAIN_BACKWARD, s);
      k_plain_backward<ET, PH><<<grid, 256, 0, s>>>(A, w.Ke, w.Fe);
      trace_end(KID_PLAIN_BACKWARD, s);
      FOLGB_LAUNCH_CHECK();
      return (int)FOLGB_OK;
    }
  });
  if (rc) return rc;
  if (dloss_ddofs || dloss_dcontrol) {
    rc = launch_gather(p, B, w.g, w.rec, elem_ctrl ? 0 : 1, w.scale, dloss_ddofs, (int64_t)p->ndof * p->N,
                       elem_ctrl ? nullptr : dloss_dcontrol, p->N, elem_ctrl ? dloss_dcontrol : nullptr,
                       (elem_ctrl && p->phys.loss_exponent != 1.0) ? 1 : 0, s, nullptr, nullptr);
  }
  return rc;
}

extern "C" int folgb_assemble(const folgb_plan* p, const float* control, const float* dofs, int32_t transpose,
                              float* residual, float* csr_values, float* inv_diag, int32_t* device_status,
                              void* workspace, size_t workspace_bytes, void* stream) {
  if (!p || !control || !dofs) return FOLGB_ERR_INVALID_ARGUMENT;
  if ((csr_values || inv_diag) && !p->has_csr) return FOLGB_ERR_NO_PATTERN;
  float *g, *Ke;
  size_t need = layout_assemble(p, workspace, workspace_bytes, &g, &Ke);
  if (!workspace || workspace_bytes < need) return FOLGB_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  LossWS w{g, residual_record(p), nullptr, nullptr, nullptr, nullptr, nullptr};
  VecArgs A = make_vec_args(p, 1, control, 0, dofs, 0, 0, w, nullptr, nullptr, device_status);
  MatArgs M;
  M.E = p->E;
  M.conn = p->d_conn;
  M.xyz4 = p->d_xyz4;
  M.gp = p->d_gp;
  M.ctrl = control;
  M.ctrl_stride = 0;
  M.dofs = dofs;
  M.dofs_stride = 0;
  M.dmask = p->d_dmask;
  M.k0 = p->d_k0;
  M.dval = p->d_dval;
  M.apply_dirichlet = 0;
  M.ctrl_layout = p->ctrl_layout;
  M.mat = p->mat;
  M.transpose = transpose ? 1 : 0;
  M.epb = 0;
  M.Ke = Ke;
  M.Fe = nullptr;
  M.g = nullptr;
  M.rec = residual_record(p);
  M.dctrl_elem = nullptr;
  M.exponent = 1.f;
  M.inv_batch = 1.f;
  M.status = device_status;
  const int npts = p->h_gp.npts;
  dim3 grid((unsigned)loss_blocks(p), 1u);
  int rc = dispatch(p->etype, p->physics, [&](auto tag) -> int {
    constexpr int ET = decltype(tag)::ET, PH = decltype(tag)::PH;
    if (residual) {
      if (!(p->phys.kernel_variant != 1 && launch_hex8_fast(p, A, grid, MODE_RESIDUAL, s))) {
        trace_begin(KID_ELEM_RESIDUAL, s);
        with_const_gp<ET>(p, [&](auto np) {
          k_elem_vector<ET, PH, MODE_RESIDUAL, false, decltype(np)::value><<<grid, 256, 0, s>>>(A, 1);
        });
        trace_end(KID_ELEM_RESIDUAL, s);
      }
      FOLGB_LAUNCH_CHECK();
    }
    if (csr_values || inv_diag) return launch_matrix<ET, PH, MAT_ASSEMBLE>(M, 1, npts, s);
    return (int)FOLGB_OK;
  });
  if (rc) return rc;
  if (residual) {
    rc = launch_gather(p, 1, g, residual_record(p), 0, nullptr, residual, 0, nullptr, 0, nullptr, 0, s, nullptr,
                       nullptr);
    if (rc) return rc;
  }
  if (csr_values || inv_diag) {
    int blocks = (int)((p->P + 255) / 256);
    int cap = num_sms() * 16;
    if (blocks > cap) blocks = cap;
    trace_begin(KID_PAIR_REDUCE, s);
    switch (p->ndof) {
      case 1:
        k_pair_reduce<1><<<blocks, 256, 0, s>>>(p->P, p->d_pair_row, p->d_adj_ptr, p->d_adj, p->d_pair_ptr,
                                                 p->d_pair_slot, p->d_rowptr, Ke, csr_values, inv_diag);
        break;
      case 2:
        k_pair_reduce<2><<<blocks, 256, 0, s>>>(p->P, p->d_pair_row, p->d_adj_ptr, p->d_adj, p->d_pair_ptr,
                                                 p->d_pair_slot, p->d_rowptr, Ke, csr_values, inv_diag);
        break;
      case 3:
        k_pair_reduce<3><<<blocks, 256, 0, s>>>(p->P, p->d_pair_row, p->d_adj_ptr, p->d_adj, p->d_pair_ptr,
                                                 p->d_pair_slot, p->d_rowptr, Ke, csr_values, inv_diag);
        break;
    }
    trace_end(KID_PAIR_REDUCE, s);
    FOLGB_LAUNCH_CHECK();
  }
  return FOLGB_OK;
}

namespace folgb {
int hex8_variant_count();
bool hex8_variant_applies(const folgb_plan* p, int v);
}

// Times every kernel variant of the plan's loss + adjoint path on the given
// inputs (2 warm-up and `repeats` timed calls each, CUDA events on the stream)
// and keeps the fastest in the plan.  With a flush buffer, each timed call is
// preceded (outside its events) by a write of the whole buffer, so the calls
// start with the mesh tables and inputs out of L2, as they do in a training
// step.  Synchronises the stream.
static int autotune_impl(folgb_plan* p, int32_t batch, const float* control, int64_t control_stride,
                         const float* dofs, int64_t dofs_stride, float* losses, float* dloss_ddofs,
                         float* dloss_dcontrol, void* workspace, size_t workspace_bytes, int32_t repeats,
                         void* stream, int32_t* chosen, float* ms_per_variant, int32_t max_variants,
                         void* flush, size_t flush_bytes) {
  if (!p || !chosen) return FOLGB_ERR_INVALID_ARGUMENT;
  const bool tunable = p->etype == FOLGB_HEX8 && p->physics == FOLGB_ELASTIC && p->phys.num_gp == 2 &&
                       p->phys.kernel_variant == 0;  // a forced variant is not retuned
  const int nv = tunable ? hex8_variant_count() : 1;
  if (repeats <= 0) repeats = 5;
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t a, b;
  FOLGB_CUDA_TRY(cudaEventCreate(&a));
  FOLGB_CUDA_TRY(cudaEventCreate(&b));
  // an untunable plan is timed as it stands (its variant, forced or not, is kept)
  int best = p->hex8_variant;
  float best_ms = 0.f;
  bool timed_any = false;
  int rc = FOLGB_OK;
  for (int v = 0; v < nv && rc == FOLGB_OK; ++v) {
    if (tunable && !hex8_variant_applies(p, v)) {  // not timed: -1
      if (ms_per_variant && v < max_variants) ms_per_variant[v] = -1.f;
      continue;
    }
    if (tunable) p->hex8_variant = v;
    for (int k = 0; k < 2 && rc == FOLGB_OK; ++k)
      rc = folgb_loss_adjoint(p, batch, control, control_stride, dofs, dofs_stride, 1, losses, dloss_ddofs,
                              dloss_dcontrol, nullptr, workspace, workspace_bytes, stream);
    float ms = 0.f;
    for (int k = 0; k < repeats && rc == FOLGB_OK; ++k) {
      if (flush && flush_bytes && cudaMemsetAsync(flush, k & 0xff, flush_bytes, s) != cudaSuccess) rc = FOLGB_ERR_CUDA;
      cudaEventRecord(a, s);
      if (rc == FOLGB_OK)
        rc = folgb_loss_adjoint(p, batch, control, control_stride, dofs, dofs_stride, 1, losses, dloss_ddofs,
                                dloss_dcontrol, nullptr, workspace, workspace_bytes, stream);
      cudaEventRecord(b, s);
      if (cudaEventSynchronize(b) != cudaSuccess) rc = FOLGB_ERR_CUDA;
      float one = 0.f;
      cudaEventElapsedTime(&one, a, b);
      ms += one;
    }
    ms /= repeats;
    if (ms_per_variant && v < max_variants) ms_per_variant[v] = ms;
    if (tunable && (!timed_any || ms < best_ms)) {
      best = v;
      best_ms = ms;
      timed_any = true;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  p->hex8_variant = best;
  *chosen = best;
  return rc;
}

extern "C" int folgb_autotune(folgb_plan* p, int32_t batch, const float* control, int64_t control_stride,
                              const float* dofs, int64_t dofs_stride, float* losses, float* dloss_ddofs,
                              float* dloss_dcontrol, void* workspace, size_t workspace_bytes, int32_t repeats,
                              void* stream, int32_t* chosen, float* ms_per_variant, int32_t max_variants) {
  return autotune_impl(p, batch, control, control_stride, dofs, dofs_stride, losses, dloss_ddofs, dloss_dcontrol,
                       workspace, workspace_bytes, repeats, stream, chosen, ms_per_variant, max_variants, nullptr, 0);
}

extern "C" int folgb_autotune_flushed(folgb_plan* p, int32_t batch, const float* control, int64_t control_stride,
                                      const float* dofs, int64_t dofs_stride, float* losses, float* dloss_ddofs,
                                      float* dloss_dcontrol, void* workspace, size_t workspace_bytes,
                                      int32_t repeats, void* stream, int32_t* chosen, float* ms_per_variant,
                                      int32_t max_variants, void* flush_buffer, size_t flush_bytes) {
  if (!flush_buffer || !flush_bytes) return FOLGB_ERR_INVALID_ARGUMENT;
  return autotune_impl(p, batch, control, control_stride, dofs, dofs_stride, losses, dloss_ddofs, dloss_dcontrol,
                       workspace, workspace_bytes, repeats, stream, chosen, ms_per_variant, max_variants,
                       flush_buffer, flush_bytes);
}
