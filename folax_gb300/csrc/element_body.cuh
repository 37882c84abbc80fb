// Per-element device code shared by the single-mesh and the batched kernels:
// argument blocks, gathers, the Gauss-point loop of each element physics,
// and the deterministic loss reduction.
//
// Reference behaviour restated here (paths inside the folax project):
//   gather by connectivity          fol/loss_functions/fe_loss.py:155-164, 232-248
//   isoparametric map               fol/geometries/geometry.py:87-97
//   thermal element                 fol/loss_functions/thermal.py:28-49
//   linear elastic element          fol/loss_functions/mechanical.py:98-117
//   Neo-Hookean (AD) element        fol/loss_functions/mechanical_neohooke_AD.py:254-293
//   split Neo-Hookean element       fol/loss_functions/mechanical_neohooke.py:243-275
//   Saint-Venant-Kirchhoff element  fol/loss_functions/mechanical_saint_venant.py:263-296
//   transient thermal element       fol/loss_functions/transient_thermal.py:43-78
//   batch loss                      fol/loss_functions/fe_loss.py:250-262
#pragma once

#include <cmath>
#include <type_traits>

#include "folgb_internal.cuh"

namespace folgb {

template <int ET_, int PH_>
struct Tag {
  static constexpr int ET = ET_, PH = PH_;
};

template <class F>
int dispatch(int et, int ph, F&& f) {
  switch (et * 6 + ph) {
    case 0: return f(Tag<FOLGB_QUAD4, FOLGB_THERMAL>{});
    case 1: return f(Tag<FOLGB_QUAD4, FOLGB_ELASTIC>{});
    case 2: return f(Tag<FOLGB_QUAD4, FOLGB_NEOHOOKE>{});
    case 3: return f(Tag<FOLGB_QUAD4, FOLGB_SAINT_VENANT>{});
    case 4: return f(Tag<FOLGB_QUAD4, FOLGB_TRANSIENT_THERMAL>{});
    case 5: return f(Tag<FOLGB_QUAD4, FOLGB_NEOHOOKE_SPLIT>{});
    case 6: return f(Tag<FOLGB_HEX8, FOLGB_THERMAL>{});
    case 7: return f(Tag<FOLGB_HEX8, FOLGB_ELASTIC>{});
    case 8: return f(Tag<FOLGB_HEX8, FOLGB_NEOHOOKE>{});
    case 9: return f(Tag<FOLGB_HEX8, FOLGB_SAINT_VENANT>{});
    case 10: return f(Tag<FOLGB_HEX8, FOLGB_TRANSIENT_THERMAL>{});
    case 11: return f(Tag<FOLGB_HEX8, FOLGB_NEOHOOKE_SPLIT>{});
    case 12: return f(Tag<FOLGB_TET4, FOLGB_THERMAL>{});
    case 13: return f(Tag<FOLGB_TET4, FOLGB_ELASTIC>{});
    case 14: return f(Tag<FOLGB_TET4, FOLGB_NEOHOOKE>{});
    case 15: return f(Tag<FOLGB_TET4, FOLGB_SAINT_VENANT>{});
    case 16: return f(Tag<FOLGB_TET4, FOLGB_TRANSIENT_THERMAL>{});
    case 17: return f(Tag<FOLGB_TET4, FOLGB_NEOHOOKE_SPLIT>{});
  }
  return FOLGB_ERR_INVALID_ARGUMENT;
}

enum { MODE_LOSS = 0, MODE_RESIDUAL = 1 };

// Calls f(std::integral_constant<int, NP>) with the plan's compile-time Gauss
// rule (const_gp_points), instantiating only the rules element type ET has.
template <int ET, class F>
void with_const_gp(const folgb_plan* p, F&& f) {
  const int np = const_gp_points(p->etype, p->phys.num_gp);
  if constexpr (ET == FOLGB_QUAD4) {
    if (np == 4) return f(std::integral_constant<int, 4>{});
  } else if constexpr (ET == FOLGB_TET4) {
    if (np == 1) return f(std::integral_constant<int, 1>{});
  }
  f(std::integral_constant<int, 0>{});
}

struct VecArgs {
  int64_t E, N;
  const int* conn;
  const float4* xyz4;
  const GPTable* gp;
  const float* ctrl;
  int64_t ctrl_stride;
  const float* dofs;
  int64_t dofs_stride;
  const unsigned char* dmask;
  const unsigned char* elem_bc;  // [E] element touches a Dirichlet dof
  const float* k0;               // [N] nodal material field (transient thermal)
  const float* dval;
  int apply_dirichlet;
  int ctrl_layout;
  MatConst mat;
  // element results: one record of `rec` floats per (instance, element, node)
  // = ndof vector components (+ the nodal control sensitivity), local-node-major:
  // record (b, e, a) starts at ((b*nen + a)*E + e)*rec
  float* g;
  int rec;
  float* dctrl_elem;  // [B][E] element-layout control gradient or NULL
  float* partials;    // [B][gridDim.x]
  unsigned* counters; // [B]
  float* losses;      // [B]
  float* scale;       // [B]
  float exponent, inv_batch;
  int* status;
  int stream_rec = 0;  // 1: records larger than L2; store them evict-first (__stcs)
  // tile-local kernels write the finished nodes' gradients themselves
  float* out = nullptr;          // [B][out_stride] dLoss/d dofs
  int64_t out_stride = 0;
  float* dctrl_nodal = nullptr;  // [B][N] nodal control gradient (nodal layout)
};

__device__ __forceinline__ void load_gp_table(GPTable& dst, const GPTable* src) {
  const int* s = reinterpret_cast<const int*>(src);
  int* d = reinterpret_cast<int*>(&dst);
  // npts first, then only the rows that are used
  for (int i = threadIdx.x; i < (int)(sizeof(GPTable) / 4); i += blockDim.x) d[i] = __ldg(s + i);
}

template <int NEN>
__device__ __forceinline__ void load_nodes(const int* conn, int64_t e, int (&nodes)[NEN]) {
  if constexpr (NEN == 8) {
    const int4* c4 = reinterpret_cast<const int4*>(conn + e * 8);
    int4 p = __ldg(c4), q = __ldg(c4 + 1);
    nodes[0] = p.x; nodes[1] = p.y; nodes[2] = p.z; nodes[3] = p.w;
    nodes[4] = q.x; nodes[5] = q.y; nodes[6] = q.z; nodes[7] = q.w;
  } else {
    int4 p = __ldg(reinterpret_cast<const int4*>(conn + e * 4));
    nodes[0] = p.x; nodes[1] = p.y; nodes[2] = p.z; nodes[3] = p.w;
  }
}

// Last-block-done reduction of per-block energies into the per-instance loss:
// the block that finishes last (integer atomic counter) sums the partials in
// a fixed order, so the result is deterministic.
__device__ __forceinline__ void finish_loss(float block_energy, const VecArgs& A, int b, float* sh) {
  __shared__ bool last;
  const int nblk = gridDim.x;
  if (threadIdx.x == 0) {
    A.partials[(int64_t)b * nblk + blockIdx.x] = block_energy;
    __threadfence();
    unsigned prev = atomicAdd(A.counters + b, 1u);
    last = (prev == (unsigned)nblk - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  float s = 0.f;
  const volatile float* pv = A.partials + (int64_t)b * nblk;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) s += pv[i];
  float L = block_sum(s, sh);
  if (threadIdx.x == 0) {
    float p = A.exponent;
    float Lp = (p == 1.f) ? L : powf(L, p);
    float sc = (p == 1.f) ? A.inv_batch : p * powf(L, p - 1.f) * A.inv_batch;
    A.losses[b] = Lp;
    A.scale[b] = sc;
    if (!isfinite(Lp) && A.status) atomicOr(A.status, 1 << FOLGB_ERR_NAN);
    A.counters[b] = 0u;  // ready for the next launch
  }
}

// One record store of up to 4 floats at float offset off of A.g (records are
// 1, 2 or 4 floats, padding zeroed); evict-first when the records do not fit
// in L2, so they do not push the node data out of it.
__device__ __forceinline__ void store_record(const VecArgs& A, int64_t off, const float (&v)[4]) {
  float* rec = A.g + off;
  if (A.rec == 4) {
    const float4 t = make_float4(v[0], v[1], v[2], v[3]);
    if (A.stream_rec) __stcs(reinterpret_cast<float4*>(rec), t);
    else *reinterpret_cast<float4*>(rec) = t;
  } else if (A.rec == 2) {
    const float2 t = make_float2(v[0], v[1]);
    if (A.stream_rec) __stcs(reinterpret_cast<float2*>(rec), t);
    else *reinterpret_cast<float2*>(rec) = t;
  } else if (A.rec == 3) {  // unpadded 3-component records (tet patches)
    if (A.stream_rec) {
      __stcs(rec, v[0]);
      __stcs(rec + 1, v[1]);
      __stcs(rec + 2, v[2]);
    } else {
      rec[0] = v[0];
      rec[1] = v[1];
      rec[2] = v[2];
    }
  } else {
    if (A.stream_rec) __stcs(rec, v[0]);
    else rec[0] = v[0];
  }
}

// The element body with its per-node results handed to sink(a, v): v holds
// the ndof vector components of local node a, then the nodal control
// sensitivity (nodal controls, loss mode), zero padded to 4.
template <int ET, int PH, int MODE, int NP, class Sink>
__device__ __forceinline__ void elem_vector_body_to(const VecArgs& A, const GPTable& gp, const int b, const int64_t e,
                                                    float& energy, int& bad, Sink&& sink) {
  constexpr int NEN = ElemT<ET>::NEN, DIM = ElemT<ET>::DIM, NDOF = NdofT<PH, DIM>::V;
  constexpr int ND = NEN * NDOF;
  {
    int nodes[NEN];
    load_nodes<NEN>(A.conn, e, nodes);
    float X[NEN][3];
    float ue[ND];
    float de[NEN];
    float ke[PH == FOLGB_TRANSIENT_THERMAL ? NEN : 1];
    float eval = 0.f;
    const float* dofs = A.dofs + (int64_t)b * A.dofs_stride;
    const float* ctrl = A.ctrl + (int64_t)b * A.ctrl_stride;
    const bool bc = A.apply_dirichlet && __ldg(A.elem_bc + e);
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
      float4 x = __ldg(A.xyz4 + nodes[a]);
      X[a][0] = x.x; X[a][1] = x.y; X[a][2] = x.z;
      unsigned m = bc ? __ldg(A.dmask + nodes[a]) : 0u;
#pragma unroll
      for (int c = 0; c < NDOF; ++c) {
        int64_t d = (int64_t)NDOF * nodes[a] + c;
        ue[a * NDOF + c] = ((m >> c) & 1u) ? __ldg(A.dval + d) : __ldg(dofs + d);
      }
      if (A.ctrl_layout == FOLGB_CONTROL_NODAL) de[a] = __ldg(ctrl + nodes[a]);
      if constexpr (PH == FOLGB_TRANSIENT_THERMAL) ke[a] = __ldg(A.k0 + nodes[a]);
    }
    if (A.ctrl_layout != FOLGB_CONTROL_NODAL) eval = __ldg(ctrl + e);
    float g[ND];
    float gd[NEN];
#pragma unroll
    for (int i = 0; i < ND; ++i) g[i] = 0.f;
#pragma unroll
    for (int a = 0; a < NEN; ++a) gd[a] = 0.f;
    const MatConst& mt = A.mat;
    auto point = [&](const int q) {
      float J[DIM][DIM];
#pragma unroll
      for (int i = 0; i < DIM; ++i)
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
          float s = 0.f;
#pragma unroll
          for (int a = 0; a < NEN; ++a) s = fmaf(X[a][i], dN_at<ET, NP>(gp, q, a, k), s);
          J[i][k] = s;
        }
      float Ji[DIM][DIM];
      float det = det_inv<DIM>(J, Ji);
      bad |= !(det > 0.f);
      const float wd = gp_w<ET, NP>(gp, q) * det;
      // dN/dx = dN/dxi J^-1; the transient thermal element uses J^-1 dN/dxi^T
      // instead (transient_thermal.py:57-59), the same for symmetric J
      constexpr bool kTransposedInverse = PH == FOLGB_TRANSIENT_THERMAL;
      float dNdx[NEN][DIM];
#pragma unroll
      for (int a = 0; a < NEN; ++a)
#pragma unroll
        for (int j = 0; j < DIM; ++j) {
          float s = 0.f;
#pragma unroll
          for (int k = 0; k < DIM; ++k) s = fmaf(dN_at<ET, NP>(gp, q, a, k), kTransposedInverse ? Ji[j][k] : Ji[k][j], s);
          dNdx[a][j] = s;
        }
      float egp;
      if (A.ctrl_layout == FOLGB_CONTROL_NODAL) {
        egp = 0.f;
#pragma unroll
        for (int a = 0; a < NEN; ++a) egp = fmaf(gp_N<ET, NP>(gp, q, a), de[a], egp);
      } else {
        egp = eval;
      }
      if constexpr (PH == FOLGB_THERMAL) {
        float Tg = 0.f, gT[DIM];
#pragma unroll
        for (int j = 0; j < DIM; ++j) gT[j] = 0.f;
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
          Tg = fmaf(gp_N<ET, NP>(gp, q, a), ue[a], Tg);
#pragma unroll
          for (int j = 0; j < DIM; ++j) gT[j] = fmaf(ue[a], dNdx[a][j], gT[j]);
        }
        float gf = 1.f;
        if (mt.beta != 0.f) gf = 1.f + mt.beta * powf(Tg, mt.c);
        float kw = wd * egp * gf;
        float gg = 0.f;
#pragma unroll
        for (int j = 0; j < DIM; ++j) gg = fmaf(gT[j], gT[j], gg);
        energy = fmaf(kw, gg, energy);
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
          float s = 0.f;
#pragma unroll
          for (int j = 0; j < DIM; ++j) s = fmaf(dNdx[a][j], gT[j], s);
          g[a] = fmaf(kw, s, g[a]);
          gd[a] = fmaf(wd * gf * gg, gp_N<ET, NP>(gp, q, a), gd[a]);
        }
      } else if constexpr (PH == FOLGB_ELASTIC) {
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
        }
        float sig[DIM][DIM];
#pragma unroll
        for (int i = 0; i < DIM; ++i) {
          sig[i][i] = egp * (mt.lam * tr + 2.f * mt.mu * H[i][i]);
#pragma unroll
          for (int j = i + 1; j < DIM; ++j) {
            float gam = H[i][j] + H[j][i];
            sh2 = fmaf(gam, gam, sh2);
            sig[i][j] = sig[j][i] = egp * mt.mu * gam;
          }
        }
        float sed = mt.lam * tr * tr + 2.f * mt.mu * sq + mt.mu * sh2;
        energy = fmaf(wd * egp, sed, energy);
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
#pragma unroll
          for (int i = 0; i < DIM; ++i) {
            float s = 0.f;
#pragma unroll
            for (int j = 0; j < DIM; ++j) s = fmaf(sig[i][j], dNdx[a][j], s);
            g[a * DIM + i] = fmaf(wd, s, g[a * DIM + i]);
          }
          gd[a] = fmaf(wd * sed, gp_N<ET, NP>(gp, q, a), gd[a]);
        }
        if (mt.has_bf) {
#pragma unroll
          for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int i = 0; i < DIM; ++i) {
              float f = wd * gp_N<ET, NP>(gp, q, a) * mt.bf[i];
              g[a * DIM + i] -= f;
              energy = fmaf(-f, ue[a * DIM + i], energy);
            }
        }
      } else if constexpr (PH == FOLGB_TRANSIENT_THERMAL) {
        // egp is the current temperature at the point (the nodal control)
        float Tn = 0.f, kq = 0.f, gT[DIM];
#pragma unroll
        for (int j = 0; j < DIM; ++j) gT[j] = 0.f;
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
          Tn = fmaf(gp_N<ET, NP>(gp, q, a), ue[a], Tn);
          kq = fmaf(gp_N<ET, NP>(gp, q, a), ke[a], kq);
#pragma unroll
          for (int j = 0; j < DIM; ++j) gT[j] = fmaf(ue[a], dNdx[a][j], gT[j]);
        }
        const float Kc = kq * (1.f + mt.mbeta * powf(Tn, mt.c));
        const float dKdT = kq * mt.mbeta * mt.c * powf(Tn, mt.c - 1.f);
        float gg = 0.f;
#pragma unroll
        for (int j = 0; j < DIM; ++j) gg = fmaf(gT[j], gT[j], gg);
        const float diff = Tn - egp, rc = mt.rho_cp;
        energy = fmaf(wd, 0.5f * Kc * gg + 0.5f * rc / mt.dt * diff * diff, energy);
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
          float gn = 0.f;
#pragma unroll
          for (int j = 0; j < DIM; ++j) gn = fmaf(dNdx[a][j], gT[j], gn);
          if (MODE == MODE_LOSS) {
            g[a] = fmaf(wd, Kc * gn + (0.5f * dKdT * gg + rc / mt.dt * diff) * gp_N<ET, NP>(gp, q, a), g[a]);
            gd[a] = fmaf(-wd * rc / mt.dt * diff, gp_N<ET, NP>(gp, q, a), gd[a]);
          } else {
            g[a] = fmaf(wd, rc * diff * gp_N<ET, NP>(gp, q, a) + mt.dt * Kc * gn, g[a]);
          }
        }
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
        NHSState<DIM> st;
        nh_split_state<DIM>(H, mt.kap_f * egp, mt.mu_f * egp, st);
        float P[DIM][DIM];  // first Piola-Kirchhoff stress F S
#pragma unroll
        for (int k = 0; k < DIM; ++k)
#pragma unroll
          for (int j = 0; j < DIM; ++j) {
            float s = 0.f;
#pragma unroll
            for (int p = 0; p < DIM; ++p) s = fmaf(st.F[k][p], st.S[p][j], s);
            P[k][j] = s;
          }
        energy = fmaf(wd, st.psi, energy);
        const float dpsi_de = st.dpsi_dk * mt.kap_f + st.dpsi_dmu * mt.mu_f;
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
#pragma unroll
          for (int k = 0; k < DIM; ++k) {
            float s = 0.f;
#pragma unroll
            for (int j = 0; j < DIM; ++j) s = fmaf(P[k][j], dNdx[a][j], s);
            g[a * DIM + k] = fmaf(wd, s, g[a * DIM + k]);
          }
          gd[a] = fmaf(wd * dpsi_de, gp_N<ET, NP>(gp, q, a), gd[a]);
        }
        if (MODE == MODE_RESIDUAL && mt.has_bf) {
#pragma unroll
          for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int i = 0; i < DIM; ++i) g[a * DIM + i] -= wd * gp_N<ET, NP>(gp, q, a) * mt.bf[i];
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
        SVKState<DIM> st;
        svk_state<DIM>(H, mt.mu_f * egp, mt.lam_f * egp, mt.mu_f, mt.lam_f, st);
        float P[DIM][DIM];  // first Piola-Kirchhoff stress F S
#pragma unroll
        for (int k = 0; k < DIM; ++k)
#pragma unroll
          for (int j = 0; j < DIM; ++j) {
            float s = 0.f;
#pragma unroll
            for (int p = 0; p < DIM; ++p) s = fmaf(st.F[k][p], st.S[p][j], s);
            P[k][j] = s;
          }
        energy = fmaf(wd, st.psi, energy);
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
#pragma unroll
          for (int k = 0; k < DIM; ++k) {
            float s = 0.f;
#pragma unroll
            for (int j = 0; j < DIM; ++j) s = fmaf(P[k][j], dNdx[a][j], s);
            g[a * DIM + k] = fmaf(wd, s, g[a * DIM + k]);
          }
          gd[a] = fmaf(wd * st.dpsi_de, gp_N<ET, NP>(gp, q, a), gd[a]);
        }
        if (MODE == MODE_RESIDUAL && mt.has_bf) {
#pragma unroll
          for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int i = 0; i < DIM; ++i) g[a * DIM + i] -= wd * gp_N<ET, NP>(gp, q, a) * mt.bf[i];
        }
      } else {  // neo-Hooke
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
        float P[DIM][DIM];
        float psi, dpsi_dmu, dpsi_dlam;
        if constexpr (MODE == MODE_LOSS) {
          // the loss gradient is the true dpsi/dF
          nh_first_piola<DIM>(H, mu, lam, P, psi, dpsi_dmu, dpsi_dlam);
        } else {
          // the FE residual: F S, the shear entries of S doubled in the
          // reference convention
          NHState<DIM> st;
          nh_state<DIM>(H, mu, lam, st);
          float M[DIM][DIM];
          const float off = mt.shear_ref ? 2.f : 1.f;
#pragma unroll
          for (int i = 0; i < DIM; ++i)
#pragma unroll
            for (int j = 0; j < DIM; ++j) M[i][j] = st.S[i][j] * (i == j ? 1.f : off);
#pragma unroll
          for (int k = 0; k < DIM; ++k)
#pragma unroll
            for (int j = 0; j < DIM; ++j) {
              float s = 0.f;
#pragma unroll
              for (int p = 0; p < DIM; ++p) s = fmaf(st.F[k][p], M[p][j], s);
              P[k][j] = s;
            }
          psi = st.psi;
          dpsi_dmu = st.dpsi_dmu;
          dpsi_dlam = st.dpsi_dlam;
        }
        energy = fmaf(wd, psi, energy);
        const float dpsi_de = dpsi_dmu * mt.mu_f + dpsi_dlam * mt.lam_f;
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
#pragma unroll
          for (int k = 0; k < DIM; ++k) {
            float s = 0.f;
#pragma unroll
            for (int j = 0; j < DIM; ++j) s = fmaf(P[k][j], dNdx[a][j], s);
            g[a * DIM + k] = fmaf(wd, s, g[a * DIM + k]);
          }
          gd[a] = fmaf(wd * dpsi_de, gp_N<ET, NP>(gp, q, a), gd[a]);
        }
        if (MODE == MODE_RESIDUAL && mt.has_bf) {
#pragma unroll
          for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int i = 0; i < DIM; ++i) g[a * DIM + i] -= wd * gp_N<ET, NP>(gp, q, a) * mt.bf[i];
        }
      }
    };
    if constexpr (NP > 0) {
#pragma unroll
      for (int q = 0; q < NP; ++q) point(q);
    } else {
#pragma unroll 1
      for (int q = 0; q < gp.npts; ++q) point(q);
    }
    if (!isfinite(energy)) bad |= 2;
    const bool nodal_gde = (MODE == MODE_LOSS) && A.ctrl_layout == FOLGB_CONTROL_NODAL;
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
      float v[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int c = 0; c < NDOF; ++c) v[c] = g[a * NDOF + c];
      if (nodal_gde) v[NDOF < 4 ? NDOF : 3] = gd[a];
      sink(a, v);
    }
    if (MODE == MODE_LOSS) {
      if (!nodal_gde && A.dctrl_elem) {
        float s = 0.f;
#pragma unroll
        for (int a = 0; a < NEN; ++a) s += gd[a];
        // scale by 1/B here when the exponent is 1; otherwise the gather pass rescales
        A.dctrl_elem[(int64_t)b * A.E + e] = (A.exponent == 1.f) ? s * A.inv_batch : s;
      }
    }
  }
}

// Per-element body shared by the single-mesh and the batched kernels: one
// record per (element, node), local-node-major ([b][a][e]), one vector store
// each.  NP > 0: the Gauss rule is the compile-time one of GPc (unrolled
// point loop).
template <int ET, int PH, int MODE, int NP = 0>
__device__ __forceinline__ void elem_vector_body(const VecArgs& A, const GPTable& gp, const int b, const int64_t e,
                                                 float& energy, int& bad) {
  constexpr int NEN = ElemT<ET>::NEN;
  elem_vector_body_to<ET, PH, MODE, NP>(A, gp, b, e, energy, bad, [&](int a, const float (&v)[4]) {
    store_record(A, (((int64_t)b * NEN + a) * A.E + e) * A.rec, v);
  });
}

// __syncthreads_or returns whether any thread's predicate is non-zero (not
// the bitwise OR), so each flag gets its own reduction.
// Warp-level variants of the epilogue: no block barrier, so warps that finish
// early do not wait for the slowest warp of their block.
__device__ __forceinline__ void report_bad_warp(int bad, int* status) {
  const unsigned detj = __any_sync(0xffffffffu, bad & 1), nan = __any_sync(0xffffffffu, bad & 2);
  if ((threadIdx.x & 31) == 0 && status && (detj || nan))
    atomicOr(status, (detj ? 1 << FOLGB_ERR_NONPOSITIVE_DETJ : 0) | (nan ? 1 << FOLGB_ERR_NAN : 0));
}

// Loss epilogue without barriers: each warp adds its 32 energies with a fixed
// shuffle tree and posts the sum in shared memory; the last warp of the block
// to post (a shared counter) adds the block's warp sums in warp order and
// posts the block sum; the last block (a global counter) adds the block sums
// in block order.  The order of every sum is fixed, whichever warp or block
// finishes last.  wcount must be zeroed before any warp can post.
__device__ __forceinline__ void finish_loss_warp(float energy, int bad, const VecArgs& A, int b, float* wsum,
                                                 unsigned* wcount, int blk = -1, int nblk_arg = -1) {
  report_bad_warp(bad, A.status);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) energy += __shfl_xor_sync(0xffffffffu, energy, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // the block's index among the instance's blocks (default: blockIdx.x of gridDim.x)
  const int nblk = nblk_arg >= 0 ? nblk_arg : (int)gridDim.x;
  const int bi = blk >= 0 ? blk : (int)blockIdx.x;
  int last = 0;
  if (lane == 0) {
    wsum[warp] = energy;
    __threadfence_block();
    last = atomicAdd(wcount, 1u) == (unsigned)nw - 1;
  }
  if (!__shfl_sync(0xffffffffu, last, 0)) return;
  __threadfence_block();
  float v = (lane < nw) ? ((volatile float*)wsum)[lane] : 0.f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  last = 0;
  if (lane == 0) {
    A.partials[(int64_t)b * nblk + bi] = v;
    __threadfence();
    last = atomicAdd(A.counters + b, 1u) == (unsigned)nblk - 1;
  }
  if (!__shfl_sync(0xffffffffu, last, 0)) return;
  __threadfence();
  float s = 0.f;
  const volatile float* pv = A.partials + (int64_t)b * nblk;
  for (int i = lane; i < nblk; i += 32) s += pv[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    const float p = A.exponent;
    const float Lp = (p == 1.f) ? s : powf(s, p);
    const float sc = (p == 1.f) ? A.inv_batch : p * powf(s, p - 1.f) * A.inv_batch;
    A.losses[b] = Lp;
    A.scale[b] = sc;
    if (!isfinite(Lp) && A.status) atomicOr(A.status, 1 << FOLGB_ERR_NAN);
    A.counters[b] = 0u;  // ready for the next launch
  }
}

__device__ __forceinline__ void report_bad(int bad, int* status) {
  const int detj = __syncthreads_or(bad & 1);
  const int nan = __syncthreads_or(bad & 2);
  if (threadIdx.x == 0 && status) {
    if (detj) atomicOr(status, 1 << FOLGB_ERR_NONPOSITIVE_DETJ);
    if (nan) atomicOr(status, 1 << FOLGB_ERR_NAN);
  }
}

}  // namespace folgb

namespace folgb {
// sum-factorised hex8 2x2x2 elasticity (hex8_fused.cu); returns 1 if launched
int launch_hex8_fast(const folgb_plan* p, const VecArgs& A, dim3 grid, int mode, cudaStream_t s);
int launch_tile_boundary(const folgb_plan* p, const VecArgs& A, int B, cudaStream_t s, int pdl);
// tetrahedra in patches of 6 (tet_patch.cu): loss + adjoint records per
// (instance, patch, patch node); returns 1 if launched, 0 if it does not
// apply, or the negated error code
int launch_tet_patch(const folgb_plan* p, const VecArgs& A, int B, cudaStream_t s);
// record width of the patch records: 3 unpadded floats with element controls
// (no nodal control sensitivity to carry), else the loss record
inline int tet_patch_record(const folgb_plan* p) {
  return (p->ndof == 3 && p->ctrl_layout == FOLGB_CONTROL_ELEMENT) ? 3 : loss_record(p);
}
}  // namespace folgb
