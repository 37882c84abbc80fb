// Adjoint sensitivities of an integral response (FiniteElementResponse,
// fol/responses/fe_response.py:17-526) for the thermal and small-strain
// elastic elements.
//
// Response: J = sum_e sum_q w_q detJ_q f(d_q, u_q), with d_q = N_q . d_e the
// control and u_q = N_q u_e the dofs at the Gauss point (fe_response.py:
// 92-120), and f a polynomial given as monomials c * d^p * prod_i u_i^q_i (the
// host parses the reference's formula string into them).
//
// One element kernel produces, per (element, local node), whatever is asked:
//   value        the element's share of J (block partials, last block sums);
//   rhs record   dJ/du_a                               (fe_response.py:244-283)
//   sens record  [dJ/dx_a + l.dR/dx_a, dJ/dd_a + l.dR/dd_a]  (:365-406, :486-526)
// where R is the element residual and l the adjoint dofs.  The derivatives of
// R are analytic: for elasticity l.R = sum_q w detJ d_q (grad l : C : grad u)
// - l.F, for the thermal element l.R = sum_q w detJ d_q g(T) grad l . grad T,
// and moving node a by dx_k changes detJ by detJ dN_a/dx_k and grad v by
// -(grad v)[:, k] (x) dN_a/dx.  A deterministic node gather (ascending element
// order per node) assembles the records.
#include <cmath>

#include "element_body.cuh"

namespace folgb {

constexpr int kMaxMonomials = 16;

struct RespArgs {
  int64_t E, N;
  const int* conn;
  const float4* xyz4;
  const float* ctrl;
  const float* dofs;
  const float* adj;
  int ctrl_layout;
  MatConst mat;
  int nmono;
  float coeff[kMaxMonomials];
  int dpow[kMaxMonomials];
  int upow[kMaxMonomials][3];
  float* rhs_rec;     // [nen][E][ndof] or null
  float4* sens_rec;   // [nen][E] (dx, dy, dz, dd) or null
  float* dctrl_elem;  // [E] element-layout control derivative or null
  float* partials;    // [gridDim.x] or null (value)
  unsigned* counter;
  float* value;
};

__device__ __forceinline__ float ipow(float x, int p) {
  float r = 1.f;
  for (int i = 0; i < p; ++i) r *= x;
  return r;
}

// f(d, u) and its partial derivatives
template <int NDOF>
__device__ __forceinline__ void eval_poly(const RespArgs& A, float d, const float (&u)[NDOF], float& f, float& fd,
                                          float (&fu)[NDOF]) {
  f = 0.f;
  fd = 0.f;
#pragma unroll
  for (int i = 0; i < NDOF; ++i) fu[i] = 0.f;
  for (int k = 0; k < A.nmono; ++k) {
    const int p = A.dpow[k];
    float base = A.coeff[k];
    float up[NDOF];
#pragma unroll
    for (int i = 0; i < NDOF; ++i) up[i] = ipow(u[i], A.upow[k][i]);
    float prod = 1.f;
#pragma unroll
    for (int i = 0; i < NDOF; ++i) prod *= up[i];
    f = fmaf(base * ipow(d, p), prod, f);
    if (p > 0) fd = fmaf(base * (float)p * ipow(d, p - 1), prod, fd);
#pragma unroll
    for (int i = 0; i < NDOF; ++i) {
      const int q = A.upow[k][i];
      if (q == 0) continue;
      float others = 1.f;
#pragma unroll
      for (int j = 0; j < NDOF; ++j)
        if (j != i) others *= up[j];
      fu[i] = fmaf(base * ipow(d, p) * (float)q * ipow(u[i], q - 1), others, fu[i]);
    }
  }
}

template <int ET, int PH>
__global__ void __launch_bounds__(128) k_response(const RespArgs A, const GPTable* __restrict__ gp_dev) {
  constexpr int NEN = ElemT<ET>::NEN, DIM = ElemT<ET>::DIM, NDOF = NdofT<PH, DIM>::V;
  __shared__ GPTable gp;
  __shared__ float red[32];
  __shared__ bool last;
  load_gp_table(gp, gp_dev);
  __syncthreads();
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float val = 0.f;
  if (e < A.E) {
    int nodes[NEN];
    load_nodes<NEN>(A.conn, e, nodes);
    float X[NEN][3], ue[NEN][NDOF], le[NEN][NDOF], de[NEN];
    const bool want_sens = A.sens_rec != nullptr || A.dctrl_elem != nullptr;
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
      const float4 x = __ldg(A.xyz4 + nodes[a]);
      X[a][0] = x.x;
      X[a][1] = x.y;
      X[a][2] = x.z;
#pragma unroll
      for (int c = 0; c < NDOF; ++c) {
        ue[a][c] = __ldg(A.dofs + (int64_t)NDOF * nodes[a] + c);
        le[a][c] = want_sens ? __ldg(A.adj + (int64_t)NDOF * nodes[a] + c) : 0.f;
      }
      de[a] = A.ctrl_layout == FOLGB_CONTROL_NODAL ? __ldg(A.ctrl + nodes[a]) : 0.f;
    }
    const float d_elem = A.ctrl_layout == FOLGB_CONTROL_NODAL ? 0.f : __ldg(A.ctrl + e);
    float grhs[NEN][NDOF], gx[NEN][3], gdd[NEN];
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
#pragma unroll
      for (int c = 0; c < NDOF; ++c) grhs[a][c] = 0.f;
      gx[a][0] = gx[a][1] = gx[a][2] = 0.f;
      gdd[a] = 0.f;
    }
    const MatConst& mt = A.mat;
#pragma unroll 1
    for (int q = 0; q < gp.npts; ++q) {
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
      const float wd = gp.w[q] * det;
      float G[NEN][DIM];
#pragma unroll
      for (int a = 0; a < NEN; ++a)
#pragma unroll
        for (int j = 0; j < DIM; ++j) {
          float s = 0.f;
#pragma unroll
          for (int k = 0; k < DIM; ++k) s = fmaf(dN_at<ET>(gp, q, a, k), Ji[k][j], s);
          G[a][j] = s;
        }
      float dq = d_elem;
      if (A.ctrl_layout == FOLGB_CONTROL_NODAL) {
        dq = 0.f;
#pragma unroll
        for (int a = 0; a < NEN; ++a) dq = fmaf(gp.N[q][a], de[a], dq);
      }
      float uq[NDOF];
#pragma unroll
      for (int c = 0; c < NDOF; ++c) {
        float s = 0.f;
#pragma unroll
        for (int a = 0; a < NEN; ++a) s = fmaf(gp.N[q][a], ue[a][c], s);
        uq[c] = s;
      }
      float f, fd, fu[NDOF];
      eval_poly<NDOF>(A, dq, uq, f, fd, fu);
      val = fmaf(wd, f, val);
#pragma unroll
      for (int a = 0; a < NEN; ++a) {
#pragma unroll
        for (int c = 0; c < NDOF; ++c) grhs[a][c] = fmaf(wd * fu[c], gp.N[q][a], grhs[a][c]);
        gdd[a] = fmaf(wd * fd, gp.N[q][a], gdd[a]);
#pragma unroll
        for (int k = 0; k < DIM; ++k) gx[a][k] = fmaf(wd * f, G[a][k], gx[a][k]);
      }
      if (!want_sens) continue;
      // adjoint-weighted residual l.R at this point and its derivatives
      if constexpr (PH == FOLGB_ELASTIC) {
        float Hu[DIM][DIM], Hl[DIM][DIM];
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
          for (int j = 0; j < DIM; ++j) {
            float su = 0.f, sl = 0.f;
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
              su = fmaf(ue[a][i], G[a][j], su);
              sl = fmaf(le[a][i], G[a][j], sl);
            }
            Hu[i][j] = su;
            Hl[i][j] = sl;
          }
        // sigma1(v) = lam tr(grad v) I + mu (grad v + grad v^T)  (unit control)
        float Su[DIM][DIM], Sl[DIM][DIM];
        float tru = 0.f, trl = 0.f;
#pragma unroll
        for (int i = 0; i < DIM; ++i) {
          tru += Hu[i][i];
          trl += Hl[i][i];
        }
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
          for (int j = 0; j < DIM; ++j) {
            Su[i][j] = mt.mu * (Hu[i][j] + Hu[j][i]) + (i == j ? mt.lam * tru : 0.f);
            Sl[i][j] = mt.mu * (Hl[i][j] + Hl[j][i]) + (i == j ? mt.lam * trl : 0.f);
          }
        float psi = 0.f;  // grad l : C : grad u
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
          for (int j = 0; j < DIM; ++j) psi = fmaf(Su[i][j], Hl[i][j], psi);
        float lb = 0.f;  // body force . l at the point
        if (mt.has_bf) {
#pragma unroll
          for (int i = 0; i < DIM; ++i) {
            float s = 0.f;
#pragma unroll
            for (int a = 0; a < NEN; ++a) s = fmaf(gp.N[q][a], le[a][i], s);
            lb = fmaf(mt.bf[i], s, lb);
          }
        }
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
          gdd[a] = fmaf(wd * psi, gp.N[q][a], gdd[a]);
          // d(grad v)/dx_{a,k} = -(grad v)[:, k] (x) dN_a/dx
          float SuG[DIM], SlG[DIM];
#pragma unroll
          for (int i = 0; i < DIM; ++i) {
            float s1 = 0.f, s2 = 0.f;
#pragma unroll
            for (int j = 0; j < DIM; ++j) {
              s1 = fmaf(Su[i][j], G[a][j], s1);
              s2 = fmaf(Sl[i][j], G[a][j], s2);
            }
            SuG[i] = s1;
            SlG[i] = s2;
          }
#pragma unroll
          for (int k = 0; k < DIM; ++k) {
            float dpsi = 0.f;
#pragma unroll
            for (int i = 0; i < DIM; ++i) dpsi = fmaf(Hl[i][k], SuG[i], fmaf(Hu[i][k], SlG[i], dpsi));
            gx[a][k] = fmaf(wd * dq, psi * G[a][k] - dpsi, gx[a][k]);
            if (mt.has_bf) gx[a][k] = fmaf(-wd * lb, G[a][k], gx[a][k]);
          }
        }
      } else {  // thermal
        float Tq = 0.f, gT[DIM], gl[DIM];
#pragma unroll
        for (int j = 0; j < DIM; ++j) gT[j] = gl[j] = 0.f;
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
          Tq = fmaf(gp.N[q][a], ue[a][0], Tq);
#pragma unroll
          for (int j = 0; j < DIM; ++j) {
            gT[j] = fmaf(ue[a][0], G[a][j], gT[j]);
            gl[j] = fmaf(le[a][0], G[a][j], gl[j]);
          }
        }
        const float gf = (mt.beta != 0.f) ? 1.f + mt.beta * powf(Tq, mt.c) : 1.f;
        float lT = 0.f;
#pragma unroll
        for (int j = 0; j < DIM; ++j) lT = fmaf(gl[j], gT[j], lT);
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
          gdd[a] = fmaf(wd * gf * lT, gp.N[q][a], gdd[a]);
          float GT = 0.f, Gl = 0.f;
#pragma unroll
          for (int j = 0; j < DIM; ++j) {
            GT = fmaf(G[a][j], gT[j], GT);
            Gl = fmaf(G[a][j], gl[j], Gl);
          }
#pragma unroll
          for (int k = 0; k < DIM; ++k)
            gx[a][k] = fmaf(wd * dq * gf, lT * G[a][k] - gl[k] * GT - gT[k] * Gl, gx[a][k]);
        }
      }
    }
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
      if (A.rhs_rec) {
#pragma unroll
        for (int c = 0; c < NDOF; ++c) A.rhs_rec[((int64_t)a * A.E + e) * NDOF + c] = grhs[a][c];
      }
      if (A.sens_rec) A.sens_rec[(int64_t)a * A.E + e] = make_float4(gx[a][0], gx[a][1], gx[a][2], gdd[a]);
    }
    if (A.dctrl_elem) {
      float s = 0.f;
#pragma unroll
      for (int a = 0; a < NEN; ++a) s += gdd[a];
      A.dctrl_elem[e] = s;  // element layout: N sums to one, so dd_e = sum_a dd_a
    }
  }
  if (!A.value) return;
  const float bv = block_sum(val, red);
  if (threadIdx.x == 0) {
    A.partials[blockIdx.x] = bv;
    __threadfence();
    last = atomicAdd(A.counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  float s = 0.f;
  const volatile float* pv = A.partials;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += pv[i];
  const float tot = block_sum(s, red);
  if (threadIdx.x == 0) {
    *A.value = tot;
    *A.counter = 0u;
  }
}

// node gather of NC-component records [nen][E][NC] (record index a*E + e):
// out[NC*n + c] = sign * sum over the node's incidences, zero on Dirichlet dofs
// when mask is given; out_last (optional) receives component NC-1 instead.
template <int NC>
__global__ void __launch_bounds__(256) k_response_gather(int64_t N, const int* __restrict__ inc_ptr,
                                                         const int* __restrict__ inc_slot,
                                                         const float* __restrict__ rec,
                                                         const unsigned char* __restrict__ mask, float sign,
                                                         int ncomp_out, float* __restrict__ out,
                                                         float* __restrict__ out_last) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float acc[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) acc[c] = 0.f;
  for (int k = __ldg(inc_ptr + n); k < __ldg(inc_ptr + n + 1); ++k) {
    const int64_t r = __ldg(inc_slot + k);
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] += __ldg(rec + r * NC + c);
  }
  const unsigned m = mask ? __ldg(mask + n) : 0u;
  for (int c = 0; c < ncomp_out; ++c) out[(int64_t)ncomp_out * n + c] = ((m >> c) & 1u) ? 0.f : sign * acc[c];
  if (out_last) out_last[n] = sign * acc[NC - 1];
}

struct RespWS {
  float* rhs_rec;
  float4* sens_rec;
  float* partials;
  unsigned* counter;
};

static int response_blocks(const folgb_plan* p) { return (int)((p->E + 127) / 128); }

static size_t layout_response(const folgb_plan* p, void* base, size_t cap, RespWS* w) {
  Bump bp(base, cap);
  RespWS t;
  t.rhs_rec = bp.take<float>((size_t)p->nen * p->E * p->ndof);
  t.sens_rec = bp.take<float4>((size_t)p->nen * p->E);
  t.partials = bp.take<float>((size_t)response_blocks(p));
  t.counter = bp.take<unsigned>(1);
  if (w) *w = t;
  return align_up(bp.off);
}

}  // namespace folgb

using namespace folgb;

extern "C" size_t folgb_response_workspace_bytes(const folgb_plan* p) {
  return p ? layout_response(p, nullptr, 0, nullptr) : 0;
}

extern "C" int folgb_response(const folgb_plan* p, int32_t num_monomials, const folgb_monomial* monomials,
                              const float* control, const float* dofs, const float* adjoint, float* value,
                              float* adjoint_rhs, float* dcontrol, float* dxyz, void* workspace,
                              size_t workspace_bytes, void* stream) {
  if (!p || !control || !dofs || num_monomials < 0 || num_monomials > kMaxMonomials ||
      (num_monomials > 0 && !monomials))
    return FOLGB_ERR_INVALID_ARGUMENT;
  if (is_hyperelastic(p->physics) || p->physics == FOLGB_TRANSIENT_THERMAL) return FOLGB_ERR_INVALID_ARGUMENT;
  if ((dcontrol || dxyz) && !adjoint) return FOLGB_ERR_INVALID_ARGUMENT;
  RespWS w;
  const size_t need = layout_response(p, workspace, workspace_bytes, &w);
  if (!workspace || workspace_bytes < need) return FOLGB_ERR_WORKSPACE;
  RespArgs A{};
  A.E = p->E;
  A.N = p->N;
  A.conn = p->d_conn;
  A.xyz4 = p->d_xyz4;
  A.ctrl = control;
  A.dofs = dofs;
  A.adj = adjoint;
  A.ctrl_layout = p->ctrl_layout;
  A.mat = p->mat;
  A.nmono = num_monomials;
  for (int k = 0; k < num_monomials; ++k) {
    A.coeff[k] = (float)monomials[k].coeff;
    A.dpow[k] = monomials[k].control_power;
    for (int i = 0; i < 3; ++i) A.upow[k][i] = monomials[k].dof_power[i];
    if (A.dpow[k] < 0 || A.upow[k][0] < 0 || A.upow[k][1] < 0 || A.upow[k][2] < 0) return FOLGB_ERR_INVALID_ARGUMENT;
  }
  const bool elem_ctrl = p->ctrl_layout == FOLGB_CONTROL_ELEMENT;
  A.rhs_rec = adjoint_rhs ? w.rhs_rec : nullptr;
  A.sens_rec = (dxyz || (dcontrol && !elem_ctrl)) ? w.sens_rec : nullptr;
  A.dctrl_elem = (dcontrol && elem_ctrl) ? dcontrol : nullptr;
  A.partials = w.partials;
  A.counter = w.counter;
  A.value = value;
  cudaStream_t s = (cudaStream_t)stream;
  if (value) FOLGB_CUDA_TRY(cudaMemsetAsync(w.counter, 0, sizeof(unsigned), s));
  int rc = dispatch(p->etype, p->physics, [&](auto tag) -> int {
    constexpr int ET = decltype(tag)::ET, PH = decltype(tag)::PH;
    if constexpr (is_hyperelastic(PH) || PH == FOLGB_TRANSIENT_THERMAL) {
      return FOLGB_ERR_INVALID_ARGUMENT;
    } else {
      k_response<ET, PH><<<response_blocks(p), 128, 0, s>>>(A, p->d_gp);
      FOLGB_LAUNCH_CHECK();
      return FOLGB_OK;
    }
  });
  if (rc) return rc;
  const int gb = (int)((p->N + 255) / 256);
  if (adjoint_rhs) {
    // -(dJ/du) with zeros on Dirichlet dofs (fe_response.py:270-279)
    switch (p->ndof) {
      case 1:
        k_response_gather<1><<<gb, 256, 0, s>>>(p->N, p->d_inc_ptr, p->d_inc_slot, w.rhs_rec, p->d_dmask, -1.f, 1,
                                                adjoint_rhs, nullptr);
        break;
      case 2:
        k_response_gather<2><<<gb, 256, 0, s>>>(p->N, p->d_inc_ptr, p->d_inc_slot, w.rhs_rec, p->d_dmask, -1.f, 2,
                                                adjoint_rhs, nullptr);
        break;
      default:
        k_response_gather<3><<<gb, 256, 0, s>>>(p->N, p->d_inc_ptr, p->d_inc_slot, w.rhs_rec, p->d_dmask, -1.f, 3,
                                                adjoint_rhs, nullptr);
    }
    FOLGB_LAUNCH_CHECK();
  }
  if (A.sens_rec) {
    // shape derivatives [3N] (no Dirichlet masking) and nodal control derivatives
    k_response_gather<4><<<gb, 256, 0, s>>>(p->N, p->d_inc_ptr, p->d_inc_slot,
                                            reinterpret_cast<const float*>(w.sens_rec), nullptr, 1.f, dxyz ? 3 : 0,
                                            dxyz, (dcontrol && !elem_ctrl) ? dcontrol : nullptr);
    FOLGB_LAUNCH_CHECK();
  }
  return FOLGB_OK;
}
