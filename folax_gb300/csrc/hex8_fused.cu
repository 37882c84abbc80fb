// Fused loss + adjoint for trilinear hexahedra with the 2x2x2 Gauss rule,
// linear elasticity (fol/loss_functions/mechanical.py:98-117 with
// hexahedra_3d_8.py:22-33), by sum factorisation over the element's tensor
// product structure.  Valid for any (distorted) hexahedron.
//
// A trilinear field f = sum_a f_a N_a is c0 + c1 xi + c2 eta + c3 zeta +
// c4 xi eta + c5 eta zeta + c6 xi zeta + c7 xi eta zeta; the coefficients are
// a 3-D Walsh-Hadamard butterfly of the nodal values (24 add/sub).  At Gauss
// points (xi, eta, zeta) = g (t_xi, t_eta, t_zeta), g = 1/sqrt(3):
//   df/dxi   = c1 + c4 eta + c6 zeta + c7 eta zeta   (depends on t_eta, t_zeta)
// so each reference derivative takes 4 distinct values over the 8 points:
// 12 numbers per field instead of 8 x 3 dot products of length 8.  The
// residual r_a = sum_q dN_a/dxi_k(q) T_q[k] (T = w detJ sigma J^-T) is the
// adjoint of the same map: per-direction sums over the shared points, the
// adjoint butterfly, and the transposed Hadamard transform.
//
// Node order (hexahedra_3d_8.py:79-87) -> lexicographic (xi fastest):
//   lex = [0, 1, 3, 2, 4, 5, 7, 6]   (node 2 is (+,+,-), node 3 is (-,+,-), ...)
#include <algorithm>
#include <atomic>
#include <type_traits>
#include <vector>

#include "element_body.cuh"

namespace folgb {

constexpr float kG = 0.57735026918962576f;   // 1/sqrt(3)
constexpr float kG2 = 0.33333333333333333f;  // g^2

// forward Hadamard: h[b] = sum_L f[L] prod_d s_{L,d}^{b_d}, lexicographic L and b
__device__ __forceinline__ void wht8(float (&f)[8]) {
#pragma unroll
  for (int st = 1; st < 8; st <<= 1) {
#pragma unroll
    for (int L = 0; L < 8; ++L)
      if (!(L & st)) {
        const float a = f[L], b = f[L + st];
        f[L] = a + b;       // coefficient without this axis
        f[L + st] = b - a;  // coefficient with this axis
      }
  }
}

// transposed Hadamard: r[L] = sum_b d[b] prod_d s_{L,d}^{b_d}
__device__ __forceinline__ void wht8_t(float (&d)[8]) {
#pragma unroll
  for (int st = 1; st < 8; st <<= 1) {
#pragma unroll
    for (int L = 0; L < 8; ++L)
      if (!(L & st)) {
        const float a = d[L], b = d[L + st];
        d[L] = a - b;       // node with s = -1 on this axis
        d[L + st] = a + b;  // node with s = +1
      }
  }
}

// Values at the 8 Gauss points (lexicographic) of a trilinear field given at
// the 8 nodes (lexicographic); self-adjoint, so it also maps Gauss-point
// weights to nodal sums  sum_q N_a(q) w_q.
__device__ __forceinline__ void interp8(float (&f)[8]) {
  const float p = 0.5f * (1.f + kG), m = 0.5f * (1.f - kG);
#pragma unroll
  for (int st = 1; st < 8; st <<= 1) {
#pragma unroll
    for (int L = 0; L < 8; ++L)
      if (!(L & st)) {
        const float a = f[L], b = f[L + st];
        f[L] = fmaf(p, a, m * b);
        f[L + st] = fmaf(m, a, p * b);
      }
  }
}

// 12 reference derivatives of a field from its Hadamard coefficients h:
// dxi[t_eta + 2 t_zeta], deta[t_xi + 2 t_zeta], dzeta[t_xi + 2 t_eta]
// (t = 0 for the -g point, 1 for +g); includes the 1/8 of the expansion.
struct Deriv12 {
  float dxi[4], deta[4], dzeta[4];
};

__device__ __forceinline__ void butterfly4(float A, float B, float C, float D, float (&v)[4]) {
  // v(ta, tb) = A + sa B + sb C + sa sb D, index ta + 2 tb
  const float pp = A + B, pm = A - B, qp = C + D, qm = C - D;
  v[0] = pm - qm;  // (-,-)
  v[1] = pp - qp;  // (+,-)
  v[2] = pm + qm;  // (-,+)
  v[3] = pp + qp;  // (+,+)
}

__device__ __forceinline__ void deriv12(const float (&h)[8], Deriv12& d) {
  const float s = 0.125f, sg = 0.125f * kG, sg2 = 0.125f * kG2;
  // lex b: 1 xi, 2 eta, 3 xi eta, 4 zeta, 5 xi zeta, 6 eta zeta, 7 xi eta zeta
  butterfly4(s * h[1], sg * h[3], sg * h[5], sg2 * h[7], d.dxi);
  butterfly4(s * h[2], sg * h[3], sg * h[6], sg2 * h[7], d.deta);
  butterfly4(s * h[4], sg * h[5], sg * h[6], sg2 * h[7], d.dzeta);
}

// adjoint of butterfly4: (A, B, C, D) += sum over v with the same signs
__device__ __forceinline__ void butterfly4_t(const float (&v)[4], float& A, float& B, float& C, float& D) {
  const float pm = v[0] + v[2], pp = v[1] + v[3];  // grouped by sa
  const float qm = v[2] - v[0], qp = v[3] - v[1];  // sb-weighted
  A += pp + pm;
  B += pp - pm;
  C += qp + qm;
  D += qp - qm;
}

// ---- packed fp32 pairs (Blackwell FFMA2/FMUL2/FADD2: two IEEE fp32 operations
// per instruction, each rounded as the scalar one).  ACC 2 runs the Gauss
// points in pairs (t_xi = 0, 1 at the same t_eta, t_zeta), so every per-point
// operation issues once for two points.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f), a); }  // exact a - b
// a*b - c*d with the scalar expression's rounding: fl(fl(a*b) - fl(c*d))
__device__ __forceinline__ float2 cross2(float2 a, float2 b, float2 c, float2 d) { return sub2(mul2(a, b), mul2(c, d)); }

// inverse and determinant of a pair of 3x3 matrices (the operations of det_inv<3>)
__device__ __forceinline__ float2 det_inv_pair(const float2 (&J)[3][3], float2 (&Ji)[3][3]) {
  const float2 c00 = cross2(J[1][1], J[2][2], J[1][2], J[2][1]);
  const float2 c01 = cross2(J[1][2], J[2][0], J[1][0], J[2][2]);
  const float2 c02 = cross2(J[1][0], J[2][1], J[1][1], J[2][0]);
  const float2 det = add2(add2(mul2(J[0][0], c00), mul2(J[0][1], c01)), mul2(J[0][2], c02));
  const float2 r = make_float2(1.0f / det.x, 1.0f / det.y);
  Ji[0][0] = mul2(c00, r);
  Ji[1][0] = mul2(c01, r);
  Ji[2][0] = mul2(c02, r);
  Ji[0][1] = mul2(cross2(J[0][2], J[2][1], J[0][1], J[2][2]), r);
  Ji[1][1] = mul2(cross2(J[0][0], J[2][2], J[0][2], J[2][0]), r);
  Ji[2][1] = mul2(cross2(J[0][1], J[2][0], J[0][0], J[2][1]), r);
  Ji[0][2] = mul2(cross2(J[0][1], J[1][2], J[0][2], J[1][1]), r);
  Ji[1][2] = mul2(cross2(J[0][2], J[1][0], J[0][0], J[1][2]), r);
  Ji[2][2] = mul2(cross2(J[0][0], J[1][1], J[0][1], J[1][0]), r);
  return det;
}

// Kernel variants (chosen per plan by the autotuner in launch_hex8_fast):
//   ACC 0: keep the 36 per-direction point sums, adjoint butterflies at the end;
//   ACC 1: accumulate the dual Hadamard coefficients point by point
//          (21 accumulators instead of 36: fewer registers, ~14% more adds);
//   ACC 2: as ACC 0 with the Gauss points in packed fp32 pairs;
//   BLOCK: threads per block; the register cap is 128 (512 resident threads
//          per SM) through __launch_bounds__, or REGS for the
//          k_hex8_elastic_regs wrapper: each SM sub-partition holds 16,384
//          registers, so 96 registers give 5 resident warps per partition
//          (20 per SM) and 80 give 6 (24 per SM), at the price of spills;
//   TMA:   the persistent k_hex8_elastic_tma below (connectivity streamed
//          into shared memory by bulk copies), 4 or 5 blocks per SM.
// The element math on gathered values: X and U are the coordinates and
// displacements at the 8 nodes in lexicographic order (LEX), egp the nodal
// controls (CL nodal, lexicographic) or the element control (egp[0]).  Adds
// the element energy to `energy`; g gets the residual (adjoint) per
// lexicographic node, wsed the Gauss-point weights w detJ sed (nodal
// controls), sedsum sum_q w detJ sed (element control); bad gets bit 0 for a
// non-positive detJ.  X and U are overwritten (transformed in place).
template <int CL, bool BF, int ACC>
__device__ __forceinline__ void hex8_elastic_core(const MatConst& mt, float (&X)[3][8], float (&U)[3][8],
                                                  float (&egp)[CL == FOLGB_CONTROL_NODAL ? 8 : 1], float& energy,
                                                  float& sedsum, float (&wsed)[CL == FOLGB_CONTROL_NODAL ? 8 : 1],
                                                  float (&g)[8][3], int& bad) {
  {
    float bfe = 0.f;  // u . b at the nodes, weighted below (body force only)
    float ub[BF ? 8 : 1];
    if constexpr (BF) {
#pragma unroll
      for (int L = 0; L < 8; ++L) ub[L] = U[0][L] * mt.bf[0] + U[1][L] * mt.bf[1] + U[2][L] * mt.bf[2];
    }
    // reference derivatives of the geometry and of the displacement
    // (ACC 2 forms the coordinate derivatives only for non-affine elements)
    Deriv12 DX[ACC == 2 ? 1 : 3], DU[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      wht8(X[i]);
      if constexpr (ACC != 2) deriv12(X[i], DX[i]);
      wht8(U[i]);
      deriv12(U[i], DU[i]);
    }
    float S[ACC != 1 ? 3 : 1][3][4];   // ACC 0 / 2: per-direction point sums
    float Dd[ACC == 1 ? 3 : 1][8];     // ACC 1: dual Hadamard coefficients (raw)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (ACC != 1) {
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int t = 0; t < 4; ++t) S[i][k][t] = 0.f;
      } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) Dd[i][k] = 0.f;
      }
    }
    float wdet[BF ? 8 : 1];
    if constexpr (ACC == 2) {
      // Gauss points in pairs q = (0|1) + 2 ty + 4 tz: dxi is shared by the pair,
      // deta / dzeta and every per-point quantity are packed (t_xi = 0, 1)
      float2 en2 = f2(0.f), sed2sum = f2(0.f);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int t = 0; t < 4; ++t) S[i][k][t] = 0.f;
      // Affine element (a parallelepiped, e.g. every cell of a structured box
      // mesh): the coordinates' Hadamard coefficients of xi eta, xi zeta,
      // eta zeta and xi eta zeta are zero, so deriv12 would give every point
      // the same reference derivatives (s h1, s h2, s h4: the butterflies add
      // and subtract zeros) and J is the same at all 8 points.  J^-1 and detJ
      // are then formed once from those values; the points see exactly the J,
      // J^-1 and detJ of the general path, so the results are bit-identical.
      bool affine = true;
#pragma unroll
      for (int i = 0; i < 3; ++i)
        affine &= (X[i][3] == 0.f) & (X[i][5] == 0.f) & (X[i][6] == 0.f) & (X[i][7] == 0.f);
      auto pairs = [&](auto aff) {
        constexpr bool AFF = decltype(aff)::value;
        float2 JiA[3][3], wdA;
        Deriv12 DXg[AFF ? 1 : 3];
        if constexpr (AFF) {
          constexpr float s8 = 0.125f;
          float2 J[3][3];
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            J[i][0] = f2(s8 * X[i][1]);
            J[i][1] = f2(s8 * X[i][2]);
            J[i][2] = f2(s8 * X[i][4]);
          }
          wdA = det_inv_pair(J, JiA);
          bad |= !(wdA.x > 0.f);
        } else {
#pragma unroll
          for (int i = 0; i < 3; ++i) deriv12(X[i], DXg[i]);
        }
#pragma unroll
      for (int pr = 0; pr < 4; ++pr) {
        const int ty = pr & 1, tz = pr >> 1;
        const int ix = ty + 2 * tz;
        float2 Gm[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          Gm[i][0] = f2(DU[i].dxi[ix]);
          Gm[i][1] = make_float2(DU[i].deta[2 * tz], DU[i].deta[2 * tz + 1]);
          Gm[i][2] = make_float2(DU[i].dzeta[2 * ty], DU[i].dzeta[2 * ty + 1]);
        }
        float2 Ji[3][3], wd;
        if constexpr (AFF) {
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) Ji[i][j] = JiA[i][j];
          wd = wdA;
        } else {
          float2 J[3][3];
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            J[i][0] = f2(DXg[i].dxi[ix]);
            J[i][1] = make_float2(DXg[i].deta[2 * tz], DXg[i].deta[2 * tz + 1]);
            J[i][2] = make_float2(DXg[i].dzeta[2 * ty], DXg[i].dzeta[2 * ty + 1]);
          }
          wd = det_inv_pair(J, Ji);  // Gauss weight 1
          bad |= !(wd.x > 0.f) | !(wd.y > 0.f);
        }
        if constexpr (BF) {
          wdet[2 * pr] = wd.x;
          wdet[2 * pr + 1] = wd.y;
        }
        float2 H[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) H[i][j] = fma2(Gm[i][2], Ji[2][j], fma2(Gm[i][1], Ji[1][j], mul2(Gm[i][0], Ji[0][j])));
        const float2 tr = add2(add2(H[0][0], H[1][1]), H[2][2]);
        const float2 g01 = add2(H[0][1], H[1][0]), g12 = add2(H[1][2], H[2][1]), g02 = add2(H[0][2], H[2][0]);
        const float2 sq = fma2(H[2][2], H[2][2], fma2(H[1][1], H[1][1], mul2(H[0][0], H[0][0])));
        const float2 gg = fma2(g02, g02, fma2(g12, g12, mul2(g01, g01)));
        const float2 sed = fma2(f2(mt.mu), gg, fma2(f2(2.f * mt.mu), sq, mul2(f2(mt.lam), mul2(tr, tr))));
        const float2 eq = (CL == FOLGB_CONTROL_NODAL) ? make_float2(egp[2 * pr], egp[2 * pr + 1]) : f2(egp[0]);
        const float2 ew = mul2(eq, wd);
        en2 = fma2(ew, sed, en2);
        if constexpr (CL == FOLGB_CONTROL_NODAL) {
          const float2 ws = mul2(wd, sed);
          wsed[2 * pr] = ws.x;
          wsed[2 * pr + 1] = ws.y;
        } else {
          sed2sum = fma2(wd, sed, sed2sum);
        }
        // w detJ sigma
        const float2 lt = mul2(mul2(ew, f2(mt.lam)), tr), tm = mul2(ew, f2(2.f * mt.mu)), sm = mul2(ew, f2(mt.mu));
        float2 sg[3][3];
        sg[0][0] = fma2(tm, H[0][0], lt);
        sg[1][1] = fma2(tm, H[1][1], lt);
        sg[2][2] = fma2(tm, H[2][2], lt);
        sg[0][1] = sg[1][0] = mul2(sm, g01);
        sg[1][2] = sg[2][1] = mul2(sm, g12);
        sg[0][2] = sg[2][0] = mul2(sm, g02);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const float2 t0 = fma2(sg[i][2], Ji[0][2], fma2(sg[i][1], Ji[0][1], mul2(sg[i][0], Ji[0][0])));
          const float2 t1 = fma2(sg[i][2], Ji[1][2], fma2(sg[i][1], Ji[1][1], mul2(sg[i][0], Ji[1][0])));
          const float2 t2 = fma2(sg[i][2], Ji[2][2], fma2(sg[i][1], Ji[2][1], mul2(sg[i][0], Ji[2][0])));
          S[i][0][ix] += t0.x + t0.y;       // dxi shared by the pair
          S[i][1][2 * tz] += t1.x;           // deta index t_xi + 2 t_zeta
          S[i][1][2 * tz + 1] += t1.y;
          S[i][2][2 * ty] += t2.x;           // dzeta index t_xi + 2 t_eta
          S[i][2][2 * ty + 1] += t2.y;
        }
      }
      };
      if (affine) pairs(std::true_type{});
      else pairs(std::false_type{});
      energy += en2.x + en2.y;
      sedsum += sed2sum.x + sed2sum.y;
    } else {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int tx = q & 1, ty = (q >> 1) & 1, tz = (q >> 2) & 1;
      const int ix = ty + 2 * tz, iy = tx + 2 * tz, iz = tx + 2 * ty;
      float J[3][3], Gm[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        J[i][0] = DX[i].dxi[ix];
        J[i][1] = DX[i].deta[iy];
        J[i][2] = DX[i].dzeta[iz];
        Gm[i][0] = DU[i].dxi[ix];
        Gm[i][1] = DU[i].deta[iy];
        Gm[i][2] = DU[i].dzeta[iz];
      }
      float Ji[3][3];
      const float det = det_inv<3>(J, Ji);
      bad |= !(det > 0.f);
      const float wd = det;  // Gauss weight 1
      if constexpr (BF) wdet[q] = wd;
      float H[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) H[i][j] = Gm[i][0] * Ji[0][j] + Gm[i][1] * Ji[1][j] + Gm[i][2] * Ji[2][j];
      const float tr = H[0][0] + H[1][1] + H[2][2];
      const float g01 = H[0][1] + H[1][0], g12 = H[1][2] + H[2][1], g02 = H[0][2] + H[2][0];
      const float sed = mt.lam * tr * tr + 2.f * mt.mu * (H[0][0] * H[0][0] + H[1][1] * H[1][1] + H[2][2] * H[2][2]) +
                        mt.mu * (g01 * g01 + g12 * g12 + g02 * g02);
      const float eq = (CL == FOLGB_CONTROL_NODAL) ? egp[q] : egp[0];
      const float ew = eq * wd;
      energy = fmaf(ew, sed, energy);
      if constexpr (CL == FOLGB_CONTROL_NODAL) wsed[q] = wd * sed;
      else sedsum = fmaf(wd, sed, sedsum);
      // w detJ sigma
      const float lt = ew * mt.lam * tr, tm = 2.f * ew * mt.mu, sm = ew * mt.mu;
      float sg[3][3];
      sg[0][0] = fmaf(tm, H[0][0], lt);
      sg[1][1] = fmaf(tm, H[1][1], lt);
      sg[2][2] = fmaf(tm, H[2][2], lt);
      sg[0][1] = sg[1][0] = sm * g01;
      sg[1][2] = sg[2][1] = sm * g12;
      sg[0][2] = sg[2][0] = sm * g02;
      const float sx = tx ? 1.f : -1.f, sy = ty ? 1.f : -1.f, sz = tz ? 1.f : -1.f;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float t0 = sg[i][0] * Ji[0][0] + sg[i][1] * Ji[0][1] + sg[i][2] * Ji[0][2];
        const float t1 = sg[i][0] * Ji[1][0] + sg[i][1] * Ji[1][1] + sg[i][2] * Ji[1][2];
        const float t2 = sg[i][0] * Ji[2][0] + sg[i][1] * Ji[2][1] + sg[i][2] * Ji[2][2];
        if (ACC == 0) {
          S[i][0][ix] += t0;
          S[i][1][iy] += t1;
          S[i][2][iz] += t2;
        } else {
          // lex b: 1 xi, 2 eta, 3 xi eta, 4 zeta, 5 xi zeta, 6 eta zeta, 7 xi eta zeta
          Dd[i][1] += t0;
          Dd[i][3] = fmaf(sy, t0, Dd[i][3]);
          Dd[i][5] = fmaf(sz, t0, Dd[i][5]);
          Dd[i][7] = fmaf(sy * sz, t0, Dd[i][7]);
          Dd[i][2] += t1;
          Dd[i][3] = fmaf(sx, t1, Dd[i][3]);
          Dd[i][6] = fmaf(sz, t1, Dd[i][6]);
          Dd[i][7] = fmaf(sx * sz, t1, Dd[i][7]);
          Dd[i][4] += t2;
          Dd[i][5] = fmaf(sx, t2, Dd[i][5]);
          Dd[i][6] = fmaf(sy, t2, Dd[i][6]);
          Dd[i][7] = fmaf(sx * sy, t2, Dd[i][7]);
        }
      }
    }
    }  // ACC != 2
    // adjoint: per component, dual Hadamard coefficients then the transposed transform
    const float s = 0.125f, sg_ = 0.125f * kG, sg2 = 0.125f * kG2;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      float d[8];
      if (ACC != 1) {
#pragma unroll
        for (int k = 0; k < 8; ++k) d[k] = 0.f;
        float A1 = 0.f, B1 = 0.f, C1 = 0.f, D1 = 0.f;
        butterfly4_t(S[i][0], A1, B1, C1, D1);  // xi: (1, xi eta, xi zeta, xi eta zeta)
        d[1] += A1;
        d[3] += B1;
        d[5] += C1;
        d[7] += D1;
        float A2 = 0.f, B2 = 0.f, C2 = 0.f, D2 = 0.f;
        butterfly4_t(S[i][1], A2, B2, C2, D2);  // eta: (eta, xi eta, eta zeta, xi eta zeta)
        d[2] += A2;
        d[3] += B2;
        d[6] += C2;
        d[7] += D2;
        float A3 = 0.f, B3 = 0.f, C3 = 0.f, D3 = 0.f;
        butterfly4_t(S[i][2], A3, B3, C3, D3);  // zeta: (zeta, xi zeta, eta zeta, xi eta zeta)
        d[4] += A3;
        d[5] += B3;
        d[6] += C3;
        d[7] += D3;
      } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) d[k] = Dd[i][k];
      }
      d[0] = 0.f;
      d[1] *= s;
      d[2] *= s;
      d[4] *= s;
      d[3] *= sg_;
      d[5] *= sg_;
      d[6] *= sg_;
      d[7] *= sg2;
      wht8_t(d);
#pragma unroll
      for (int L = 0; L < 8; ++L) g[L][i] = d[L];
    }
    if constexpr (BF) {
      interp8(wdet);  // nodal weights sum_q w detJ N_a(q)
#pragma unroll
      for (int L = 0; L < 8; ++L) {
#pragma unroll
        for (int i = 0; i < 3; ++i) g[L][i] = fmaf(-wdet[L], mt.bf[i], g[L][i]);
        bfe = fmaf(wdet[L], ub[L], bfe);
      }
      energy -= bfe;
    }
  }
}

// One element: gathers, the 8 Gauss points, the adjoint, the records.
// nodes[] are the element's node ids in the reference's local order.
template <int CL, int MODE, bool BF, int ACC>
__device__ __forceinline__ void hex8_elastic_elem(const VecArgs& A, const int b, const int64_t e,
                                                  const int (&nodes)[8], float& energy, int& bad) {
  {
    constexpr int LEX[8] = {0, 1, 3, 2, 4, 5, 7, 6};  // lex position -> node
    const float* dofs = A.dofs + (int64_t)b * A.dofs_stride;
    const float* ctrl = A.ctrl + (int64_t)b * A.ctrl_stride;
    const bool bc = A.apply_dirichlet && __ldg(A.elem_bc + e);
    float X[3][8], U[3][8];
    float egp[CL == FOLGB_CONTROL_NODAL ? 8 : 1];
#pragma unroll
    for (int L = 0; L < 8; ++L) {
      const int n = nodes[LEX[L]];
      const float4 x = __ldg(A.xyz4 + n);
      X[0][L] = x.x;
      X[1][L] = x.y;
      X[2][L] = x.z;
      const unsigned m = bc ? __ldg(A.dmask + n) : 0u;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int64_t d = 3 * (int64_t)n + c;
        U[c][L] = ((m >> c) & 1u) ? __ldg(A.dval + d) : __ldg(dofs + d);
      }
      if constexpr (CL == FOLGB_CONTROL_NODAL) egp[L] = __ldg(ctrl + n);
    }
    if constexpr (CL == FOLGB_CONTROL_NODAL) interp8(egp);
    else egp[0] = __ldg(ctrl + e);
    float wsed[CL == FOLGB_CONTROL_NODAL ? 8 : 1];
    float g[8][3];
    float sedsum = 0.f;
    hex8_elastic_core<CL, BF, ACC>(A.mat, X, U, egp, energy, sedsum, wsed, g, bad);
    if (!isfinite(energy)) bad |= 2;
    // 16-byte records, local-node-major ([b][a][e]): the 3 vector components
    // and the nodal control sensitivity (or padding); for each local node the
    // warp's stores are contiguous
    constexpr bool nodal_gde = (MODE == MODE_LOSS) && (CL == FOLGB_CONTROL_NODAL);
    if constexpr (nodal_gde) interp8(wsed);
    float4* out = reinterpret_cast<float4*>(A.g);
#pragma unroll
    for (int L = 0; L < 8; ++L) {
      float w = 0.f;
      if constexpr (nodal_gde) w = wsed[L];
      out[((int64_t)b * 8 + LEX[L]) * A.E + e] = make_float4(g[L][0], g[L][1], g[L][2], w);
    }
    if (MODE == MODE_LOSS && CL != FOLGB_CONTROL_NODAL && A.dctrl_elem)
      A.dctrl_elem[(int64_t)b * A.E + e] = (A.exponent == 1.f) ? sedsum * A.inv_batch : sedsum;
  }
}

// One element per thread.
template <int CL, int MODE, bool BF, int ACC>
__device__ __forceinline__ void hex8_elastic_body(const VecArgs& A) {
  __shared__ float wsum[32];
  __shared__ unsigned wcount;
  pdl_launch_dependents();  // the gather may start its independent loads during this kernel's tail
  if (MODE == MODE_LOSS) {
    if (threadIdx.x == 0) wcount = 0u;
    __syncthreads();
  }
  const int b = blockIdx.y;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float energy = 0.f;
  int bad = 0;
  if (e < A.E) {
    int nodes[8];
    load_nodes<8>(A.conn, e, nodes);
    hex8_elastic_elem<CL, MODE, BF, ACC>(A, b, e, nodes, energy, bad);
  }
  if constexpr (MODE == MODE_LOSS) finish_loss_warp(energy, bad, A, b, wsum, &wcount);
  else report_bad_warp(bad, A.status);
}

// Persistent variant with the connectivity streamed by the TMA engine.  Each
// warp owns a fixed, strided sequence of 32-element tiles (tiles gw, gw + W,
// ... for global warp gw of W) and keeps kTmaStages of them in flight: lane 0
// issues one bulk copy per tile (the tile's 32 connectivity rows, 1 KB) into
// the warp's stage buffer in shared memory, completing on that stage's
// mbarrier.  A tile's node gathers therefore start as soon as its rows have
// landed, with no dependent global load in front of them, and the rows of
// the next tiles arrive while this one computes.  The fixed tile order keeps
// every energy sum in a fixed order.  Every mbarrier wait is bounded: a copy
// that never lands sets FOLGB_ERR_TIMEOUT in the status word and the warp
// stops after waiting (bounded) for its other copies in flight.
constexpr int kTmaStages = 3;
constexpr int kTmaWarps = 4;  // 128 threads per block

//
// PF (prefetch): when the next tile's rows have already landed (a
// non-blocking mbarrier test), each lane prefetches its next element's node
// coordinates and dofs into L1 (PF 1) or L2 (PF 2) before computing the
// current element, so the next tile's gathers hit the cache.
template <int PF>
__device__ __forceinline__ void prefetch_node(const void* p) {
  if constexpr (PF == 1) asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
  else asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

template <int CL, int MODE, bool BF, int ACC, int PF, class Elem>
__device__ __forceinline__ void hex8_elastic_tma_body(const VecArgs& A, Elem&& elem) {
  __shared__ float wsum[32];
  __shared__ unsigned wcount;
  __shared__ __align__(128) int4 rows[kTmaWarps][kTmaStages][64];  // 32 elements x 8 node ids
  __shared__ __align__(8) uint64_t bar[kTmaWarps][kTmaStages];
  pdl_launch_dependents();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) wcount = 0u;
  if (lane == 0) {
#pragma unroll
    for (int st = 0; st < kTmaStages; ++st) mbar_init(&bar[warp][st], 1);
    fence_mbar_init();
  }
  __syncthreads();  // wcount and the barriers are initialised
  const int b = blockIdx.y;
  // element counts fit in int: folgb_plan_create bounds E * nen^2 by INT32_MAX
  const int E = (int)A.E, ntiles = (E + 31) >> 5;
  const int gw = blockIdx.x * kTmaWarps + warp, W = gridDim.x * kTmaWarps;
  auto issue = [&](int t, int st) {
    const int n = E - t * 32;
    const unsigned bytes = (unsigned)((n < 32 ? n : 32) * 32);  // whole rows: a multiple of 16
    mbar_arrive_expect_tx(&bar[warp][st], bytes);
    bulk_copy_g2s(&rows[warp][st][0], A.conn + (int64_t)t * 256, bytes, &bar[warp][st]);
  };
  if (lane == 0) {
#pragma unroll
    for (int st = 0; st < kTmaStages; ++st)
      if (gw + st * W < ntiles) issue(gw + st * W, st);
  }
  float energy = 0.f;
  int bad = 0;
  int st = 0;
  unsigned parity = 0u;
  int t = gw;
  bool timed_out = false;
  for (; t < ntiles; t += W) {
    if (!__all_sync(0xffffffffu, mbar_wait_bounded(&bar[warp][st], parity))) {
      timed_out = true;
      break;
    }
    const int e = t * 32 + lane;
    if constexpr (PF > 0) {
      const int sn = st + 1 == kTmaStages ? 0 : st + 1;
      const unsigned pn = sn == 0 ? parity ^ 1u : parity;
      const int en = (t + W) * 32 + lane;
      // the next tile's rows, only once they have landed (never waits)
      if (t + W < ntiles && en < E && mbar_test_wait(&bar[warp][sn], pn)) {
        const int4 p = rows[warp][sn][2 * lane], q = rows[warp][sn][2 * lane + 1];
        const int nn[8] = {p.x, p.y, p.z, p.w, q.x, q.y, q.z, q.w};
        const float* dofs = A.dofs + (int64_t)b * A.dofs_stride;
#pragma unroll
        for (int a = 0; a < 8; ++a) {
          prefetch_node<PF>(A.xyz4 + nn[a]);
          prefetch_node<PF>(dofs + 3 * (int64_t)nn[a]);
        }
      }
    }
    if (e < E) {
      const int4 p = rows[warp][st][2 * lane], q = rows[warp][st][2 * lane + 1];
      const int nodes[8] = {p.x, p.y, p.z, p.w, q.x, q.y, q.z, q.w};
      elem(b, e, nodes, energy, bad);
    }
    __syncwarp();  // every lane has used its rows of this stage
    if (lane == 0 && t + kTmaStages * W < ntiles) {
      fence_proxy_async_smem();
      issue(t + kTmaStages * W, st);
    }
    if (++st == kTmaStages) {
      st = 0;
      parity ^= 1u;
    }
  }
  if (timed_out && lane == 0) {
    // copies still in flight target this block's shared memory: wait for
    // them (bounded) before leaving
    for (int j = 0; j < kTmaStages; ++j) {
      if (t + j * W < ntiles) mbar_wait_bounded(&bar[warp][st], parity);
      if (++st == kTmaStages) {
        st = 0;
        parity ^= 1u;
      }
    }
    if (A.status) atomicOr(A.status, 1 << FOLGB_ERR_TIMEOUT);
  }
  if constexpr (MODE == MODE_LOSS) finish_loss_warp(energy, bad, A, b, wsum, &wcount);
  else report_bad_warp(bad, A.status);
}

template <int CL, int MODE, bool BF, int ACC, int MINB, int PF>
__global__ void __launch_bounds__(kTmaWarps * 32, MINB) k_hex8_elastic_tma(const VecArgs A) {
  hex8_elastic_tma_body<CL, MODE, BF, ACC, PF>(
      A, [&](int b, int64_t e, const int (&nodes)[8], float& energy, int& bad) {
        hex8_elastic_elem<CL, MODE, BF, ACC>(A, b, e, nodes, energy, bad);
      });
}

// ---------------------------------------------------------------------------
// Uniform box meshes (every element the same axis-aligned box; uniform_box.cu
// builds the blocks).  In the Walsh-Hadamard basis of the nodal values the
// element matrix K (energy E_e u.K u, residual E_e K u, the quadratic form of
// the pointwise evaluation above) is block diagonal: the mode (component c,
// Hadamard index b) couples only with the modes of the same reflection
// parity p = b ^ (1 << c).  Per element: the forward transform of the three
// components, eight 3 x 3 block products (72 FMA, the block entries are
// kernel parameters, read from the constant bank), the energy u.K u as the
// dot product of the transformed vectors, and the transposed transform of
// E_e K^ u^ for the residual records.  Loads, Dirichlet substitution, records
// and the element control sensitivity are those of hex8_elastic_elem
// (element controls, no body force).
template <int MODE>
__device__ __forceinline__ void box_elem(const VecArgs& A, const BoxK& K, const int b, const int64_t e,
                                         const int (&nodes)[8], float& energy, int& bad) {
  constexpr int LEX[8] = {0, 1, 3, 2, 4, 5, 7, 6};  // lex position -> node
  const float* dofs = A.dofs + (int64_t)b * A.dofs_stride;
  const bool bc = A.apply_dirichlet && __ldg(A.elem_bc + e);
  float U[3][8];
#pragma unroll
  for (int L = 0; L < 8; ++L) {
    const int n = nodes[LEX[L]];
    const unsigned m = bc ? __ldg(A.dmask + n) : 0u;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t d = 3 * (int64_t)n + c;
      U[c][L] = ((m >> c) & 1u) ? __ldg(A.dval + d) : __ldg(dofs + d);
    }
  }
  const float ee = __ldg(A.ctrl + (int64_t)b * A.ctrl_stride + e);
#pragma unroll
  for (int c = 0; c < 3; ++c) wht8(U[c]);
  float V[3][8];
#pragma unroll
  for (int p = 0; p < 8; ++p) {
    const float u0 = U[0][p ^ 1], u1 = U[1][p ^ 2], u2 = U[2][p ^ 4];
#pragma unroll
    for (int c = 0; c < 3; ++c)
      V[c][p ^ (1 << c)] = fmaf(K.k[p][c][2], u2, fmaf(K.k[p][c][1], u1, K.k[p][c][0] * u0));
  }
  float sed = 0.f;  // u.K u = sum_q detJ sed_q
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int q = 0; q < 8; ++q) sed = fmaf(U[c][q], V[c][q], sed);
  energy = fmaf(ee, sed, energy);
  if (!isfinite(energy)) bad |= 2;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
#pragma unroll
    for (int q = 0; q < 8; ++q) V[c][q] *= ee;
    wht8_t(V[c]);
  }
  float4* out = reinterpret_cast<float4*>(A.g);
#pragma unroll
  for (int L = 0; L < 8; ++L)
    out[((int64_t)b * 8 + LEX[L]) * A.E + e] = make_float4(V[0][L], V[1][L], V[2][L], 0.f);
  if (MODE == MODE_LOSS && A.dctrl_elem)
    A.dctrl_elem[(int64_t)b * A.E + e] = (A.exponent == 1.f) ? sed * A.inv_batch : sed;
}

// One box element per thread; BLOCK * MINB threads per SM (64 registers at 1,024).
template <int MODE, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) k_hex8_box(const VecArgs A, const BoxK K) {
  __shared__ float wsum[32];
  __shared__ unsigned wcount;
  pdl_launch_dependents();
  if (MODE == MODE_LOSS) {
    if (threadIdx.x == 0) wcount = 0u;
    __syncthreads();
  }
  const int b = blockIdx.y;
  const int64_t e = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  float energy = 0.f;
  int bad = 0;
  if (e < A.E) {
    int nodes[8];
    load_nodes<8>(A.conn, e, nodes);
    box_elem<MODE>(A, K, b, e, nodes, energy, bad);
  }
  if constexpr (MODE == MODE_LOSS) finish_loss_warp(energy, bad, A, b, wsum, &wcount);
  else report_bad_warp(bad, A.status);
}

// The persistent TMA-staged loop of k_hex8_elastic_tma with the box element.
template <int MODE, int MINB>
__global__ void __launch_bounds__(kTmaWarps * 32, MINB) k_hex8_box_tma(const VecArgs A, const BoxK K) {
  hex8_elastic_tma_body<FOLGB_CONTROL_ELEMENT, MODE, false, 2, 0>(
      A, [&](int b, int64_t e, const int (&nodes)[8], float& energy, int& bad) {
        box_elem<MODE>(A, K, b, e, nodes, energy, bad);
      });
}

template <int CL, int MODE, bool BF, int ACC, int BLOCK>
__global__ void __launch_bounds__(BLOCK, 512 / BLOCK) k_hex8_elastic(const VecArgs A) {
  hex8_elastic_body<CL, MODE, BF, ACC>(A);
}

template <int CL, int MODE, bool BF, int ACC, int REGS>
__global__ void __maxnreg__(REGS) k_hex8_elastic_regs(const VecArgs A) {
  hex8_elastic_body<CL, MODE, BF, ACC>(A);
}

template <int CL, int MODE, int ACC, int BLOCK>
static void launch_variant(const VecArgs& A, dim3 grid, bool bf, cudaStream_t s) {
  dim3 g2((unsigned)((A.E + BLOCK - 1) / BLOCK), grid.y);
  if (bf) k_hex8_elastic<CL, MODE, true, ACC, BLOCK><<<g2, BLOCK, 0, s>>>(A);
  else k_hex8_elastic<CL, MODE, false, ACC, BLOCK><<<g2, BLOCK, 0, s>>>(A);
}

template <int CL, int MODE, int ACC, int REGS>
static void launch_variant_regs(const VecArgs& A, dim3 grid, bool bf, cudaStream_t s) {
  dim3 g2((unsigned)((A.E + 127) / 128), grid.y);
  if (bf) k_hex8_elastic_regs<CL, MODE, true, ACC, REGS><<<g2, 128, 0, s>>>(A);
  else k_hex8_elastic_regs<CL, MODE, false, ACC, REGS><<<g2, 128, 0, s>>>(A);
}

// Resident blocks per SM of `kernel` on the current device, queried once per
// (kernel instantiation, device): cache[dev] is that instantiation's own
// table (0 = not queried yet; racing threads store the same value).
constexpr int kOccDevices = 64;
template <class K>
static int blocks_per_sm(K kernel, int threads, size_t smem, std::atomic<int> (&cache)[kOccDevices]) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kOccDevices) dev = 0;
  int n = cache[dev].load(std::memory_order_relaxed);
  if (n == 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess || n < 1) n = 1;
    cache[dev].store(n, std::memory_order_relaxed);
  }
  return n;
}

// Persistent grid: as many blocks as fit on the GPU at once, at most one
// 4-warp block per 4 tiles.
template <class K>
static unsigned persistent_blocks(K kernel, int64_t E, std::atomic<int> (&cache)[kOccDevices]) {
  const int per_sm = blocks_per_sm(kernel, kTmaWarps * 32, 0, cache);
  const int64_t want = (((E + 31) >> 5) + kTmaWarps - 1) / kTmaWarps;
  const int64_t cap = (int64_t)per_sm * num_sms();
  return (unsigned)(want < cap ? want : cap);
}

template <int CL, int MODE, int ACC, int MINB, int PF = 0>
static void launch_variant_tma(const VecArgs& A, dim3 grid, bool bf, cudaStream_t s) {
  static std::atomic<int> occ_bf[kOccDevices], occ[kOccDevices];  // per kernel instantiation and device
  if (bf) {
    auto k = k_hex8_elastic_tma<CL, MODE, true, ACC, MINB, PF>;
    k<<<dim3(persistent_blocks(k, A.E, occ_bf), grid.y), kTmaWarps * 32, 0, s>>>(A);
  } else {
    auto k = k_hex8_elastic_tma<CL, MODE, false, ACC, MINB, PF>;
    k<<<dim3(persistent_blocks(k, A.E, occ), grid.y), kTmaWarps * 32, 0, s>>>(A);
  }
}

// ---------------------------------------------------------------------------
// Structured uniform box meshes (the box mesh numbering: nodes x fastest, then
// y, then z; element (i, j, k) = i + nx (j + ny k) with the reference's local
// node order): the whole fused loss + adjoint in one launch, with no element
// records in global memory and no gather.
//
// A block owns the nodes of a column tile [x0, x0 + kGridTX) x [y0, y0 + kGridTY)
// (the last tiles also own the mesh's last node plane) and a chunk of node
// layers [z0, z1) (the nz + 1 node layers split into nzc nearly equal chunks,
// nzc chosen so the launch fills the resident blocks of the GPU in one or two
// waves), and walks the element layers z0 - 1 ... upwards.  Its
// (kGridTX + 1) x (kGridTY + 1) threads each take one element column
// (x0 - 1 + tx, y0 - 1 + ty): the elements of the halo row, column and layer
// below the tile are evaluated by this block too (they belong to the
// neighbouring tiles), so every owned node is finished here.
//
// The 8-point Hadamard transform of an element is the 4-point transform of
// each face (x and y stages) followed by the z stage, so an element column
// transforms each node layer once: the upper face of one element is the lower
// face of the next.  The residual runs the same way backwards: the
// transposed z stage splits the block products into a lower and an upper
// face part, and the upper part of layer kz - 1 is added to the lower part of
// layer kz before the one transposed face transform, which gives the element
// column's four corner contributions to node layer kz.  Per element layer:
// each thread evaluates its element (the dofs of the layer above were loaded
// one layer ahead), stores its four corner contributions in shared memory,
// and after a barrier, as node (x0 + tx, y0 + ty), adds the contributions of
// the four element columns around it in a fixed order and writes the node.
// Energies and element control gradients come from owned elements only.  The
// loss exponent must be 1 (the gradients are scaled as they are written).
constexpr int kGridTX = 16, kGridTY = 8;
constexpr int kGridCols = (kGridTX + 1) * (kGridTY + 1);  // element columns per block
constexpr int kGridBlock = (kGridCols + 31) / 32 * 32;

struct GridDims {
  int nx, ny, nz;  // elements per direction
  int zlo, zhi;    // node layers of this launch [zlo, zhi) (all: 0, nz + 1)
  int nzc;         // chunks of those layers
  int tiles_x, tiles_y;
  int blk_off, nblk;  // this launch's first block and the blocks of all launches of the step (loss sum)
  const unsigned char* layer_bc;  // [nz + 1] 1 if the node layer has a Dirichlet dof
};

// 4-point Hadamard transform of a face (lex a = ax + 2 ay), the x and y stages
// of wht8; h4t is its transpose (the x and y stages of wht8_t).
__device__ __forceinline__ void h4(float (&f)[4]) {
  float a = f[0], b = f[1];
  f[0] = a + b;
  f[1] = b - a;
  a = f[2];
  b = f[3];
  f[2] = a + b;
  f[3] = b - a;
  a = f[0];
  b = f[2];
  f[0] = a + b;
  f[2] = b - a;
  a = f[1];
  b = f[3];
  f[1] = a + b;
  f[3] = b - a;
}
__device__ __forceinline__ void h4t(float (&d)[4]) {
  float a = d[0], b = d[1];
  d[0] = a - b;
  d[1] = a + b;
  a = d[2];
  b = d[3];
  d[2] = a - b;
  d[3] = a + b;
  a = d[0];
  b = d[2];
  d[0] = a - b;
  d[2] = a + b;
  a = d[1];
  b = d[3];
  d[1] = a - b;
  d[3] = a + b;
}

// The x and y displacement components of a face travel as packed fp32 pairs
// (FADD2 / FFMA2 / FMUL2: each half rounded as the scalar operation), the z
// component as a scalar.
struct FacePair {
  float2 xy[4];
  float z[4];
};

__device__ __forceinline__ void h4p(float2 (&f)[4]) {
  float2 a = f[0], b = f[1];
  f[0] = add2(a, b);
  f[1] = sub2(b, a);
  a = f[2];
  b = f[3];
  f[2] = add2(a, b);
  f[3] = sub2(b, a);
  a = f[0];
  b = f[2];
  f[0] = add2(a, b);
  f[2] = sub2(b, a);
  a = f[1];
  b = f[3];
  f[1] = add2(a, b);
  f[3] = sub2(b, a);
}
__device__ __forceinline__ void h4tp(float2 (&d)[4]) {
  float2 a = d[0], b = d[1];
  d[0] = sub2(a, b);
  d[1] = add2(a, b);
  a = d[2];
  b = d[3];
  d[2] = sub2(a, b);
  d[3] = add2(a, b);
  a = d[0];
  b = d[2];
  d[0] = sub2(a, b);
  d[2] = add2(a, b);
  a = d[1];
  b = d[3];
  d[1] = sub2(a, b);
  d[3] = add2(a, b);
}

__global__ void __launch_bounds__(kGridBlock, 4) k_hex8_box_grid(const VecArgs A, const BoxK K, const GridDims G) {
  // corner contributions of each element column, double-buffered by layer: a
  // buffer is rewritten two layers later, after the barrier of the layer
  // between, so one barrier per layer orders the writes and the reads
  __shared__ float2 cnr_xy[2][4][kGridTY + 1][kGridTX + 1];
  __shared__ float cnr_z[2][4][kGridTY + 1][kGridTX + 1];
  __shared__ float wsum[32];
  __shared__ unsigned wcount;
  pdl_launch_dependents();
  if (threadIdx.x == 0) wcount = 0u;
  const int b = blockIdx.y;
  int t = blockIdx.x;
  const int bx = t % G.tiles_x;
  t /= G.tiles_x;
  const int by = t % G.tiles_y, bz = t / G.tiles_y;
  const int x0 = bx * kGridTX, y0 = by * kGridTY;
  const int z0 = G.zlo + (int)((int64_t)bz * (G.zhi - G.zlo) / G.nzc);
  const int NX = G.nx + 1, NXY = NX * (G.ny + 1);  // nodes per row, per layer
  // owned node counts of this tile (the last tiles own the final plane too)
  const int onx = x0 + kGridTX >= G.nx ? NX - x0 : kGridTX;
  const int ony = y0 + kGridTY >= G.ny ? G.ny + 1 - y0 : kGridTY;
  const int zend = G.zlo + (int)((int64_t)(bz + 1) * (G.zhi - G.zlo) / G.nzc);  // node layers [z0, zend)
  const bool col = threadIdx.x < kGridCols;
  const int tx = threadIdx.x % (kGridTX + 1), ty = threadIdx.x / (kGridTX + 1);
  const int ex = x0 - 1 + tx, ey = y0 - 1 + ty;
  const bool col_valid = col && ex >= 0 && ex < G.nx && ey >= 0 && ey < G.ny;
  const bool col_owned = col_valid && ex >= x0 && ey >= y0;
  const bool node_owned = col && tx < onx && ty < ony;
  const bool dir = A.apply_dirichlet != 0;
  // the element column's four nodes in a layer: n + {0, 1, NX, NX + 1}; its
  // dofs, Dirichlet mask and values advance by a layer's stride
  // 32-bit node, dof and element offsets (a grid plan has fewer than 2^31 dofs)
  const int c0 = ex + NX * ey;
  const float* dofs = A.dofs + (int64_t)b * A.dofs_stride;
  // raw dofs of a face (lex a = ax + 2 ay) and its Dirichlet mask bits (the
  // masks are read only on node layers that have a Dirichlet dof)
  auto load_face = [&](int kz, FacePair& u, unsigned& mk) {
    const int n = c0 + NXY * kz;
    mk = 0u;
    if (dir && __ldg(G.layer_bc + kz)) {
      const unsigned char* m = A.dmask + n;
      mk = (__ldg(m) & 7u) | ((__ldg(m + 1) & 7u) << 3) | ((__ldg(m + NX) & 7u) << 6) | ((__ldg(m + NX + 1) & 7u) << 9);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const float* q = dofs + 3 * (n + (a & 1) + NX * (a >> 1));
      u.xy[a] = make_float2(__ldg(q), __ldg(q + 1));
      u.z[a] = __ldg(q + 2);
    }
  };
  // Dirichlet values, then the face transform
  auto finish_face = [&](int kz, FacePair& u, unsigned mk) {
    if (mk) {
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const float* v = A.dval + 3 * (c0 + NXY * kz + (a & 1) + NX * (a >> 1));
        if ((mk >> (3 * a)) & 1u) u.xy[a].x = __ldg(v);
        if ((mk >> (3 * a + 1)) & 1u) u.xy[a].y = __ldg(v + 1);
        if ((mk >> (3 * a + 2)) & 1u) u.z[a] = __ldg(v + 2);
      }
    }
    h4p(u.xy);
    h4(u.z);
  };
  const int e0 = ex + G.nx * ey, elay = G.nx * G.ny;  // this column's element in layer 0
  const float* ctrl = A.ctrl + (int64_t)b * A.ctrl_stride;
  const int on0 = (x0 + tx) + NX * (y0 + ty);  // this thread's node in layer 0
  FacePair lo_f;            // face transform of the element's lower face (node layer kz)
  FacePair nxt;             // raw dofs of node layer kz + 1, loaded one layer ahead
  unsigned nxt_m = 0u;
  float2 hp_xy[4];          // transposed-z upper part of element layer kz - 1
  float hp_z[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    hp_xy[a] = f2(0.f);
    hp_z[a] = 0.f;
  }
  bool have_lo = false;
  float energy = 0.f;
  int bad = 0;
  auto layer_valid = [&](int kz) { return col_valid && kz >= 0 && kz < G.nz; };
  // invariant: at a valid element layer kz, nxt holds node layer kz + 1
  if (layer_valid(z0 - 1)) load_face(z0, nxt, nxt_m);
  int buf = 0;
  for (int kz = z0 - 1; kz < zend; ++kz, buf ^= 1) {
    float2 lo_xy[4], hi_xy[4];
    float lo_z[4], hi_z[4];
    if (layer_valid(kz)) {
      if (!have_lo) {  // first element of the column: its lower face
        unsigned m;
        load_face(kz, lo_f, m);
        finish_face(kz, lo_f, m);
      }
      FacePair up = nxt;
      const unsigned up_m = nxt_m;
      if (layer_valid(kz + 1)) load_face(kz + 2, nxt, nxt_m);  // the next element's upper face
      finish_face(kz + 1, up, up_m);
      const int e = e0 + elay * kz;
      const float ee = __ldg(ctrl + e);
      // z stage: Hadamard coefficients h[b] (b < 4) and h[b + 4]
      float2 Uxy[8];
      float Uz[8];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        Uxy[a] = add2(lo_f.xy[a], up.xy[a]);
        Uxy[a + 4] = sub2(up.xy[a], lo_f.xy[a]);
        Uz[a] = lo_f.z[a] + up.z[a];
        Uz[a + 4] = up.z[a] - lo_f.z[a];
      }
      lo_f = up;  // the next element's lower face
      have_lo = true;
      float2 Vxy[8];
      float Vz[8];
#pragma unroll
      for (int p = 0; p < 8; ++p) {
        const float u0 = Uxy[p ^ 1].x, u1 = Uxy[p ^ 2].y, u2 = Uz[p ^ 4];
        Vxy[p ^ 1].x = fmaf(K.k[p][0][2], u2, fmaf(K.k[p][0][1], u1, K.k[p][0][0] * u0));
        Vxy[p ^ 2].y = fmaf(K.k[p][1][2], u2, fmaf(K.k[p][1][1], u1, K.k[p][1][0] * u0));
        Vz[p ^ 4] = fmaf(K.k[p][2][2], u2, fmaf(K.k[p][2][1], u1, K.k[p][2][0] * u0));
      }
      float2 sxy = mul2(Uxy[0], Vxy[0]);
      float sz = Uz[0] * Vz[0];
#pragma unroll
      for (int q = 1; q < 8; ++q) {
        sxy = fma2(Uxy[q], Vxy[q], sxy);
        sz = fmaf(Uz[q], Vz[q], sz);
      }
      const float sed = (sxy.x + sxy.y) + sz;  // u.K u
      if (col_owned && kz >= z0) {
        energy = fmaf(ee, sed, energy);
        if (A.dctrl_elem) A.dctrl_elem[(int64_t)b * A.E + e] = sed * A.inv_batch;
      }
      if (!isfinite(sed)) bad |= 2;
      // transposed z stage of E_e K^ u^: lower (s = -1) and upper (s = +1) parts
      const float2 e2 = f2(ee);
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const float2 va = mul2(e2, Vxy[a]), vb = mul2(e2, Vxy[a + 4]);
        lo_xy[a] = sub2(va, vb);
        hi_xy[a] = add2(va, vb);
        const float za = ee * Vz[a], zb = ee * Vz[a + 4];
        lo_z[a] = za - zb;
        hi_z[a] = za + zb;
      }
    } else {
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        lo_xy[a] = hi_xy[a] = f2(0.f);
        lo_z[a] = hi_z[a] = 0.f;
      }
      have_lo = false;
      if (layer_valid(kz + 1)) load_face(kz + 2, nxt, nxt_m);  // the column starts above
    }
    // node layer kz: upper part of element layer kz - 1 + lower part of layer kz
    if (col) {
      float2 fxy[4];
      float fz[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        fxy[a] = add2(hp_xy[a], lo_xy[a]);
        fz[a] = hp_z[a] + lo_z[a];
        hp_xy[a] = hi_xy[a];
        hp_z[a] = hi_z[a];
      }
      h4tp(fxy);
      h4t(fz);
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        cnr_xy[buf][a][ty][tx] = fxy[a];
        cnr_z[buf][a][ty][tx] = fz[a];
      }
    }
    __syncthreads();
    if (node_owned && kz >= z0 && A.out) {
      // node (x0 + tx, y0 + ty): element columns (tx + ox, ty + oy), corner (1 - ox, 1 - oy)
      float2 sxy = f2(0.f);
      float sz = 0.f;
#pragma unroll
      for (int o = 0; o < 4; ++o) {
        const int ox = o & 1, oy = o >> 1;
        if (tx + ox <= kGridTX && ty + oy <= kGridTY) {
          const int a = (1 - ox) + 2 * (1 - oy);
          sxy = add2(sxy, cnr_xy[buf][a][ty + oy][tx + ox]);
          sz += cnr_z[buf][a][ty + oy][tx + ox];
        }
      }
      const int n = on0 + NXY * kz;
      const unsigned m = __ldg(G.layer_bc + kz) ? __ldg(A.dmask + n) : 0u;
      float* o = A.out + (int64_t)b * A.out_stride + 3 * n;
      o[0] = (m & 1u) ? 0.f : A.inv_batch * sxy.x;
      o[1] = (m & 2u) ? 0.f : A.inv_batch * sxy.y;
      o[2] = (m & 4u) ? 0.f : A.inv_batch * sz;
    }
  }
  finish_loss_warp(energy, bad, A, b, wsum, &wcount, G.blk_off + (int)blockIdx.x, G.nblk);
}

// ---------------------------------------------------------------------------
// Tile-local fused loss + adjoint (tiles.cu builds the tables).  One block of
// kTileElems threads per (tile, instance):
//   1. the tile's distinct nodes (coordinates, dofs with the Dirichlet values
//      substituted, nodal controls) are loaded cooperatively into shared
//      memory: one load of each node per tile instead of one per element;
//   2. each thread evaluates one element from shared memory and stores its 8
//      residual records (+ nodal control sensitivity) in shared memory,
//      corner-major so a warp's stores are conflict-free;
//   3. each local node sums its records in a fixed order; a node inside this
//      tile only writes its gradient directly, a node on the tile boundary
//      writes one partial record to global memory for k_tile_boundary.
// The element's energy goes through the fixed-order block/tile reduction.
// With a loss exponent other than 1 the gradients are written unscaled and
// k_tile_boundary scales them once the loss is known.
struct TileArgs {
  int ntiles;
  int64_t S;  // boundary slots per instance
  const int* tile_eptr;
  const int* tile_nptr;
  const int* tile_bptr;
  const int* t_elem;  // bit 31: the element touches a Dirichlet dof
  const uint2* t_lconn;
  const uint4* tn_pos;  // [K] kTileRecs record positions (uint16) of each local entry
  const int* tn_gid;
  const unsigned* tn_info;  // bits 16-18: Dirichlet mask
  const int* bn_node;
  const int* bn_ptr;
  const int* bn_slot;
  const int* in_node;
  int64_t nb_nodes, ni_nodes;
  unsigned* queue;  // [B] next tile of each instance (persistent kernel), zeroed before the launch
};

// One element of a tile from shared-memory node data: X, U (and nodal
// controls in U.w) of local nodes loc[]; Dirichlet values substituted when
// the element touches a Dirichlet dof (masks in info, node ids in gid).
// Stores the 8 residual records, corner-major, in rec; returns the energy.
template <int CL, bool BF>
__device__ __forceinline__ float tile_element(const VecArgs& A, const float* ctrl, int e_tagged, uint2 lc,
                                              const float4* sX, const float4* sU, const unsigned* info,
                                              const int* gid, float4* rec, int t, int b, int& bad) {
  constexpr int kLEX[8] = {0, 1, 3, 2, 4, 5, 7, 6};  // lex position -> reference node
  const int e = e_tagged & 0x7fffffff;
  const int loc[8] = {(int)(lc.x & 0xff), (int)((lc.x >> 8) & 0xff), (int)((lc.x >> 16) & 0xff), (int)(lc.x >> 24),
                      (int)(lc.y & 0xff), (int)((lc.y >> 8) & 0xff), (int)((lc.y >> 16) & 0xff), (int)(lc.y >> 24)};
  float X[3][8], U[3][8];
  float egp[CL == FOLGB_CONTROL_NODAL ? 8 : 1];
#pragma unroll
  for (int L = 0; L < 8; ++L) {
    const int k = loc[kLEX[L]];
    const float4 x = sX[k], u = sU[k];
    X[0][L] = x.x;
    X[1][L] = x.y;
    X[2][L] = x.z;
    U[0][L] = u.x;
    U[1][L] = u.y;
    U[2][L] = u.z;
    if constexpr (CL == FOLGB_CONTROL_NODAL) egp[L] = u.w;
  }
  if (A.apply_dirichlet && e_tagged < 0) {
#pragma unroll
    for (int L = 0; L < 8; ++L) {
      const int k = loc[kLEX[L]];
      const unsigned m = info[k] >> 16;
      if (m) {
        const int64_t d = 3 * (int64_t)gid[k];
#pragma unroll
        for (int c = 0; c < 3; ++c)
          if ((m >> c) & 1u) U[c][L] = __ldg(A.dval + d + c);
      }
    }
  }
  if constexpr (CL == FOLGB_CONTROL_NODAL) interp8(egp);
  else egp[0] = __ldg(ctrl + e);
  float wsed[CL == FOLGB_CONTROL_NODAL ? 8 : 1];
  float g[8][3];
  float sedsum = 0.f, energy = 0.f;
  hex8_elastic_core<CL, BF, 2>(A.mat, X, U, egp, energy, sedsum, wsed, g, bad);
  if (!isfinite(energy)) bad |= 2;
  if constexpr (CL == FOLGB_CONTROL_NODAL) interp8(wsed);
#pragma unroll
  for (int L = 0; L < 8; ++L) {
    float w = 0.f;
    if constexpr (CL == FOLGB_CONTROL_NODAL) w = wsed[L];
    rec[kLEX[L] * kTileElems + t] = make_float4(g[L][0], g[L][1], g[L][2], w);
  }
  if (CL != FOLGB_CONTROL_NODAL && A.dctrl_elem)
    A.dctrl_elem[(int64_t)b * A.E + e] = (A.exponent == 1.f) ? sedsum * A.inv_batch : sedsum;
  return energy;
}

// Node pass of a tile: local entry k sums its kTileRecs records (row k of
// pos; padding points at the zero record) in order, all loads issued before
// the adds; an interior node writes its gradient, an entry with partials
// (k < nb) its partial record.
template <int CL>
__device__ __forceinline__ void tile_nodes(const VecArgs& A, const float4* rec, const uint4* pos,
                                           const unsigned* info, const int* gid, int nl, int nb, float4* bpart,
                                           int b) {
  const float sc = (A.exponent == 1.f) ? A.inv_batch : 1.f;
  for (int k = threadIdx.x; k < nl; k += kTileElems) {
    const uint4 pr = pos[k];
    const unsigned w[4] = {pr.x, pr.y, pr.z, pr.w};
    float4 r[kTileRecs];
#pragma unroll
    for (int j = 0; j < kTileRecs; ++j) r[j] = rec[(w[j >> 1] >> (16 * (j & 1))) & 0xffffu];
    float4 acc = r[0];
#pragma unroll
    for (int j = 1; j < kTileRecs; ++j) {
      acc.x += r[j].x;
      acc.y += r[j].y;
      acc.z += r[j].z;
      acc.w += r[j].w;
    }
    if (k < nb) {
      bpart[k] = acc;
    } else {
      const int n = gid[k];
      const unsigned m = info[k] >> 16;
      if (A.out) {
        float* o = A.out + (int64_t)b * A.out_stride + 3 * (int64_t)n;
        o[0] = (m & 1u) ? 0.f : sc * acc.x;
        o[1] = (m & 2u) ? 0.f : sc * acc.y;
        o[2] = (m & 4u) ? 0.f : sc * acc.z;
      }
      if (CL == FOLGB_CONTROL_NODAL && A.dctrl_nodal) A.dctrl_nodal[(int64_t)b * A.N + n] = sc * acc.w;
    }
  }
}

// Simple tile kernel: one block per (tile, instance), the tile's nodes loaded
// with plain loads, then elements, then nodes.
template <int CL, bool BF, int MINB>
__global__ void __launch_bounds__(kTileElems, MINB) k_hex8_elastic_tile(const VecArgs A, const TileArgs T) {
  __shared__ float4 sX[kTileNodes];
  __shared__ float4 sU[kTileNodes];  // displacements, nodal control in w
  __shared__ unsigned sInfo[kTileNodes];
  __shared__ int sGid[kTileNodes];
  __shared__ float4 sR[8 * kTileElems + 1];  // + the zero record
  __shared__ uint4 sPos[kTileNodes];
  __shared__ float wsum[32];
  __shared__ unsigned wcount;
  pdl_launch_dependents();
  const int tile = blockIdx.x, b = blockIdx.y;
  const int e0 = __ldg(T.tile_eptr + tile), ne = __ldg(T.tile_eptr + tile + 1) - e0;
  const int n0 = __ldg(T.tile_nptr + tile), nl = __ldg(T.tile_nptr + tile + 1) - n0;
  const float* dofs = A.dofs + (int64_t)b * A.dofs_stride;
  const float* ctrl = A.ctrl + (int64_t)b * A.ctrl_stride;
  if (threadIdx.x == 0) {
    wcount = 0u;
    sR[kTileZeroRec] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  for (int k = threadIdx.x; k < nl; k += kTileElems) {
    const int n = __ldg(T.tn_gid + n0 + k);
    const float4 x = __ldg(A.xyz4 + n);
    const int64_t d = 3 * (int64_t)n;
    sX[k] = x;
    sU[k] = make_float4(__ldg(dofs + d), __ldg(dofs + d + 1), __ldg(dofs + d + 2),
                        CL == FOLGB_CONTROL_NODAL ? __ldg(ctrl + n) : 0.f);
    sInfo[k] = __ldg(T.tn_info + n0 + k);
    sGid[k] = n;
    sPos[k] = __ldg(T.tn_pos + n0 + k);
  }
  __syncthreads();
  float energy = 0.f;
  int bad = 0;
  const int t = threadIdx.x;
  if (t < ne)
    energy = tile_element<CL, BF>(A, ctrl, __ldg(T.t_elem + e0 + t), __ldg(T.t_lconn + e0 + t), sX, sU, sInfo, sGid,
                                  sR, t, b, bad);
  __syncthreads();
  const int bbase = __ldg(T.tile_bptr + tile), nb = __ldg(T.tile_bptr + tile + 1) - bbase;
  tile_nodes<CL>(A, sR, sPos, sInfo, sGid, nl, nb, reinterpret_cast<float4*>(A.g) + (int64_t)b * T.S + bbase, b);
  finish_loss_warp(energy, bad, A, b, wsum, &wcount, tile, T.ntiles);
}

// ---- persistent, pipelined tile kernel -----------------------------------
// A fixed grid of blocks per instance takes tiles from a per-instance queue
// (an atomic counter, so SMs that finish early take more tiles).  Each
// tile's inputs move into shared memory with asynchronous copies (cp.async)
// while the block computes the tile before it:
//   iteration k:  [wait for tile k's inputs]  issue the copies of tile k+1's
//   node data (ids already in shared memory) and of tile k+2's node ids,
//   elements (tile k), node pass (tile k).
// The tile's energy goes to its own partial slot (partials[tile]); the last
// block of the instance sums the slots in tile order.
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

struct TileMeta {
  int tile, e0, ne, n0, nl, bbase, nb, pad;
};

struct TileStage {
  float4 X[kTileNodes];
  float4 U[kTileNodes];
  uint4 pos[kTileNodes];
  unsigned info[kTileNodes];
  uint2 lconn[kTileElems];
  int elem[kTileElems];
};

struct TileSmem {
  TileStage st[2];
  int gid[3][kTileNodes];
  float4 rec[8 * kTileElems + 1];  // + the zero record
  TileMeta meta[4];
  float wsum[2][kTileElems / 32];
  int last;
};

__device__ __forceinline__ TileMeta tile_meta(const TileArgs& T, int tile) {
  TileMeta m{};
  m.tile = tile;
  if (tile < T.ntiles) {
    m.e0 = __ldg(T.tile_eptr + tile);
    m.ne = __ldg(T.tile_eptr + tile + 1) - m.e0;
    m.n0 = __ldg(T.tile_nptr + tile);
    m.nl = __ldg(T.tile_nptr + tile + 1) - m.n0;
    m.bbase = __ldg(T.tile_bptr + tile);
    m.nb = __ldg(T.tile_bptr + tile + 1) - m.bbase;
  }
  return m;
}

// copies of a tile's node ids (ring slot g)
__device__ __forceinline__ void issue_ids(TileSmem& S, const TileArgs& T, const TileMeta& m, int g) {
  if (m.tile >= T.ntiles) return;
  for (int k = threadIdx.x; k < m.nl; k += kTileElems) cp_async4(&S.gid[g][k], T.tn_gid + m.n0 + k);
}

// copies of a tile's inputs (node ids already in ring slot g) into stage st
template <int CL>
__device__ __forceinline__ void issue_inputs(TileSmem& S, const VecArgs& A, const TileArgs& T, const TileMeta& m,
                                             int st, int g, const float* dofs, const float* ctrl) {
  if (m.tile >= T.ntiles) return;
  TileStage& Z = S.st[st];
  for (int k = threadIdx.x; k < m.nl; k += kTileElems) {
    const int n = S.gid[g][k];
    cp_async16(&Z.X[k], A.xyz4 + n);
    const float* du = dofs + 3 * (int64_t)n;
    cp_async4(&Z.U[k].x, du);
    cp_async4(&Z.U[k].y, du + 1);
    cp_async4(&Z.U[k].z, du + 2);
    if (CL == FOLGB_CONTROL_NODAL) cp_async4(&Z.U[k].w, ctrl + n);
    cp_async4(&Z.info[k], T.tn_info + m.n0 + k);
    cp_async16(&Z.pos[k], T.tn_pos + m.n0 + k);
  }
  for (int j = threadIdx.x; j < m.ne; j += kTileElems) {
    cp_async8(&Z.lconn[j], T.t_lconn + m.e0 + j);
    cp_async4(&Z.elem[j], T.t_elem + m.e0 + j);
  }
}

template <int CL, bool BF>
__global__ void __launch_bounds__(kTileElems, 4) k_hex8_elastic_tile_pipe(const VecArgs A, const TileArgs T) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TileSmem& S = *reinterpret_cast<TileSmem*>(smem_raw);
  pdl_launch_dependents();
  const int b = blockIdx.y;
  const float* dofs = A.dofs + (int64_t)b * A.dofs_stride;
  const float* ctrl = A.ctrl + (int64_t)b * A.ctrl_stride;
  float4* bpart = reinterpret_cast<float4*>(A.g) + (int64_t)b * T.S;
  float* partials = A.partials + (int64_t)b * T.ntiles;
  // tiles k = 0, 1 of this block: blockIdx.x and gridDim.x + blockIdx.x; from
  // k = 2 on from the queue (offset by the 2 * gridDim.x tiles taken so)
  auto next_tile = [&]() { return 2 * (int)gridDim.x + (int)atomicAdd(T.queue + b, 1u); };
  if (threadIdx.x == 0) {
    S.rec[kTileZeroRec] = make_float4(0.f, 0.f, 0.f, 0.f);
    S.meta[0] = tile_meta(T, blockIdx.x);
    S.meta[1] = tile_meta(T, gridDim.x + blockIdx.x);
    S.meta[2] = tile_meta(T, S.meta[1].tile < T.ntiles ? next_tile() : T.ntiles);
  }
  __syncthreads();
  issue_ids(S, T, S.meta[0], 0);
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  issue_inputs<CL>(S, A, T, S.meta[0], 0, 0, dofs, ctrl);
  issue_ids(S, T, S.meta[1], 1);
  cp_async_commit();
  float energy_all = 0.f;  // unused beyond the flags: energies go per tile
  int bad = 0;
  for (int k = 0;; ++k) {
    const TileMeta cur = S.meta[k & 3];
    if (cur.tile >= T.ntiles) break;
    cp_async_wait<0>();  // tile k's inputs and tile k+1's ids
    __syncthreads();
    const TileMeta nx = S.meta[(k + 1) & 3], nn = S.meta[(k + 2) & 3];
    // next tile's inputs, the tile after it's ids; the tile after that from the queue
    issue_inputs<CL>(S, A, T, nx, (k + 1) & 1, (k + 1) % 3, dofs, ctrl);
    issue_ids(S, T, nn, (k + 2) % 3);
    cp_async_commit();
    if (threadIdx.x == 0) S.meta[(k + 3) & 3] = tile_meta(T, nn.tile < T.ntiles ? next_tile() : T.ntiles);
    const TileStage& Z = S.st[k & 1];
    const int t = threadIdx.x;
    float energy = 0.f;
    if (t < cur.ne)
      energy = tile_element<CL, BF>(A, ctrl, Z.elem[t], Z.lconn[t], Z.X, Z.U, Z.info, S.gid[k % 3], S.rec, t, b,
                                    bad);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) energy += __shfl_xor_sync(0xffffffffu, energy, o);
    if ((t & 31) == 0) S.wsum[k & 1][t >> 5] = energy;
    __syncthreads();
    if (t == 0) {
      float e = 0.f;
#pragma unroll
      for (int w = 0; w < kTileElems / 32; ++w) e += S.wsum[k & 1][w];
      partials[cur.tile] = e;
    }
    tile_nodes<CL>(A, S.rec, Z.pos, Z.info, S.gid[k % 3], cur.nl, cur.nb, bpart + cur.bbase, b);
  }
  cp_async_wait<0>();
  (void)energy_all;
  report_bad_warp(bad, A.status);
  // the last block of the instance sums the tile energies in tile order
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    S.last = atomicAdd(A.counters + b, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!S.last) return;
  __threadfence();
  float s = 0.f;
  const volatile float* pv = partials;
  for (int i = threadIdx.x; i < T.ntiles; i += kTileElems) s += pv[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) S.wsum[0][threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float L = 0.f;
#pragma unroll
    for (int w = 0; w < kTileElems / 32; ++w) L += S.wsum[0][w];
    const float p = A.exponent;
    const float Lp = (p == 1.f) ? L : powf(L, p);
    const float sc = (p == 1.f) ? A.inv_batch : p * powf(L, p - 1.f) * A.inv_batch;
    A.losses[b] = Lp;
    A.scale[b] = sc;
    if (!isfinite(Lp) && A.status) atomicOr(A.status, 1 << FOLGB_ERR_NAN);
    A.counters[b] = 0u;
    T.queue[b] = 0u;  // ready for the next launch
  }
}

// The nodes on tile boundaries (and nodes of no element): the partial
// records of their tiles summed in ascending tile order, scaled and written.
// With a loss exponent other than 1 it also scales what the tile kernel wrote
// unscaled (interior nodes, element control gradients).  Launched as a
// programmatic dependent of the tile kernel.
template <bool NODAL>
__global__ void __launch_bounds__(256) k_tile_boundary(const VecArgs A, const TileArgs T, int rescale) {
  const int b = blockIdx.y;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const float4* bpart = reinterpret_cast<const float4*>(A.g) + (int64_t)b * T.S;
  pdl_wait_primary();
  const float sc = (A.exponent == 1.f) ? A.inv_batch : A.scale[b];
  for (int64_t i = i0; i < T.nb_nodes; i += stride) {
    const int n = __ldg(T.bn_node + i);
    const int s0 = __ldg(T.bn_ptr + i), s1 = __ldg(T.bn_ptr + i + 1);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int j = s0; j < s1; ++j) {
      const float4 r = bpart[__ldg(T.bn_slot + j)];
      acc.x += r.x;
      acc.y += r.y;
      acc.z += r.z;
      acc.w += r.w;
    }
    if (A.out) {
      const unsigned m = __ldg(A.dmask + n);
      float* o = A.out + (int64_t)b * A.out_stride + 3 * (int64_t)n;
      o[0] = (m & 1u) ? 0.f : sc * acc.x;
      o[1] = (m & 2u) ? 0.f : sc * acc.y;
      o[2] = (m & 4u) ? 0.f : sc * acc.z;
    }
    if (NODAL && A.dctrl_nodal) A.dctrl_nodal[(int64_t)b * A.N + n] = sc * acc.w;
  }
  if (!rescale) return;
  for (int64_t i = i0; i < T.ni_nodes; i += stride) {
    const int n = __ldg(T.in_node + i);
    if (A.out) {
      float* o = A.out + (int64_t)b * A.out_stride + 3 * (int64_t)n;
      o[0] *= sc;
      o[1] *= sc;
      o[2] *= sc;
    }
    if (NODAL && A.dctrl_nodal) A.dctrl_nodal[(int64_t)b * A.N + n] *= sc;
  }
  if (!NODAL && A.dctrl_elem)
    for (int64_t e = i0; e < A.E; e += stride) A.dctrl_elem[(int64_t)b * A.E + e] *= sc;
}

static TileArgs tile_args(const folgb_plan* p) {
  TileArgs T;
  T.ntiles = p->tiles;
  T.S = p->tile_boundary_slots;
  T.tile_eptr = p->d_tile_eptr;
  T.tile_nptr = p->d_tile_nptr;
  T.tile_bptr = p->d_tile_bptr;
  T.t_elem = p->d_t_elem;
  T.t_lconn = reinterpret_cast<const uint2*>(p->d_t_lconn);
  T.tn_pos = reinterpret_cast<const uint4*>(p->d_tn_pos);
  T.tn_gid = p->d_tn_gid;
  T.tn_info = p->d_tn_info;
  T.queue = nullptr;
  T.bn_node = p->d_bn_node;
  T.bn_ptr = p->d_bn_ptr;
  T.bn_slot = p->d_bn_slot;
  T.in_node = p->d_in_node;
  T.nb_nodes = p->tile_boundary_nodes;
  T.ni_nodes = p->tile_interior_nodes;
  return T;
}

template <int CL>
static void launch_tile(const folgb_plan* p, const VecArgs& A, int B, bool bf, bool pipe, cudaStream_t s) {
  TileArgs T = tile_args(p);
  T.queue = A.counters + B;  // zeroed with the loss counters before the launch
  if (!pipe) {
    dim3 grid((unsigned)p->tiles, (unsigned)B);
    if (bf) k_hex8_elastic_tile<CL, true, 4><<<grid, kTileElems, 0, s>>>(A, T);
    else k_hex8_elastic_tile<CL, false, 4><<<grid, kTileElems, 0, s>>>(A, T);
    return;
  }
  static std::atomic<int> occ_bf[kOccDevices], occ[kOccDevices];  // per instantiation and device
  auto k = bf ? k_hex8_elastic_tile_pipe<CL, true> : k_hex8_elastic_tile_pipe<CL, false>;
  static std::atomic<int> attr_set[kOccDevices][2];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kOccDevices) dev = 0;
  if (!attr_set[dev][bf ? 1 : 0].load()) {  // more than the default 48 KB of dynamic shared memory
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TileSmem));
    attr_set[dev][bf ? 1 : 0].store(1);
  }
  const int per_sm = blocks_per_sm(k, kTileElems, sizeof(TileSmem), bf ? occ_bf : occ);
  int64_t g = (int64_t)per_sm * num_sms() / B;
  if (g > p->tiles) g = p->tiles;
  if (g < 1) g = 1;
  k<<<dim3((unsigned)g, (unsigned)B), kTileElems, sizeof(TileSmem), s>>>(A, T);
}

// Tile-local variants: kHex8TileFirst the persistent pipelined kernel,
// kHex8TileFirst + 1 the one-block-per-tile kernel.  Box variants (uniform
// box meshes): kHex8BoxFirst the persistent TMA-staged loop, then one element
// per thread in blocks of 256 and 128.
constexpr int kHex8TileFirst = 18;
constexpr int kHex8BoxFirst = 20;
constexpr int kHex8GridFirst = 23;  // structured box grid, one and two waves of blocks

// The grid kernel's tiling for `waves` waves of resident blocks over B
// instances: nzc chunks of node layers per column tile (1 <= nzc <= nz + 1).
static GridDims grid_dims(const folgb_plan* p, int B, int waves) {
  GridDims G;
  G.nx = p->box_nx;
  G.ny = p->box_ny;
  G.nz = p->box_nz;
  G.zlo = 0;
  G.zhi = G.nz + 1;
  G.tiles_x = (G.nx + kGridTX - 1) / kGridTX;
  G.tiles_y = (G.ny + kGridTY - 1) / kGridTY;
  static std::atomic<int> occ[kOccDevices];
  const int64_t slots = (int64_t)blocks_per_sm(k_hex8_box_grid, kGridBlock, 0, occ) * num_sms() * waves;
  int64_t nzc = slots / ((int64_t)G.tiles_x * G.tiles_y * B);
  if (nzc < 1) nzc = 1;
  if (nzc > G.nz + 1) nzc = G.nz + 1;
  G.nzc = (int)nzc;
  G.blk_off = 0;
  G.nblk = G.tiles_x * G.tiles_y * G.nzc;
  G.layer_bc = p->d_box_layer_bc;
  return G;
}

// most blocks per instance the grid kernel can launch (a chunk per node layer)
int64_t grid_blocks_max(const folgb_plan* p) {
  return (int64_t)((p->box_nx + kGridTX - 1) / kGridTX) * ((p->box_ny + kGridTY - 1) / kGridTY) * (p->box_nz + 1);
}

static void launch_box_grid(const folgb_plan* p, const VecArgs& A, dim3 grid, int waves, cudaStream_t s) {
  const GridDims G = grid_dims(p, (int)grid.y, waves);
  k_hex8_box_grid<<<dim3((unsigned)G.nblk, grid.y), kGridBlock, 0, s>>>(A, p->box_k, G);
}

template <int MODE>
static void launch_box(const folgb_plan* p, const VecArgs& A, dim3 grid, int variant, cudaStream_t s) {
  if (variant == kHex8BoxFirst) {
    static std::atomic<int> occ[kOccDevices];  // per instantiation and device
    auto k = k_hex8_box_tma<MODE, 6>;
    k<<<dim3(persistent_blocks(k, A.E, occ), grid.y), kTmaWarps * 32, 0, s>>>(A, p->box_k);
  } else if (variant == kHex8BoxFirst + 1) {
    k_hex8_box<MODE, 256, 4><<<dim3((unsigned)((A.E + 255) / 256), grid.y), 256, 0, s>>>(A, p->box_k);
  } else {
    k_hex8_box<MODE, 128, 8><<<dim3((unsigned)((A.E + 127) / 128), grid.y), 128, 0, s>>>(A, p->box_k);
  }
}

template <int CL, int MODE>
static void launch_cl_mode(const VecArgs& A, dim3 grid, bool bf, int variant, cudaStream_t s) {
  switch (variant) {
    case 0: launch_variant<CL, MODE, 0, 256>(A, grid, bf, s); break;
    case 1: launch_variant<CL, MODE, 0, 128>(A, grid, bf, s); break;
    case 2: launch_variant<CL, MODE, 1, 256>(A, grid, bf, s); break;
    case 3: launch_variant<CL, MODE, 1, 128>(A, grid, bf, s); break;
    case 4: launch_variant<CL, MODE, 0, 64>(A, grid, bf, s); break;
    case 5: launch_variant<CL, MODE, 1, 64>(A, grid, bf, s); break;
    case 6: launch_variant_regs<CL, MODE, 0, 96>(A, grid, bf, s); break;
    case 7: launch_variant_regs<CL, MODE, 1, 96>(A, grid, bf, s); break;
    case 8: launch_variant_regs<CL, MODE, 0, 80>(A, grid, bf, s); break;
    case 9: launch_variant_regs<CL, MODE, 1, 80>(A, grid, bf, s); break;
    case 10: launch_variant<CL, MODE, 2, 256>(A, grid, bf, s); break;
    case 11: launch_variant<CL, MODE, 2, 128>(A, grid, bf, s); break;
    case 12: launch_variant_regs<CL, MODE, 2, 96>(A, grid, bf, s); break;
    case 13: launch_variant_tma<CL, MODE, 2, 4>(A, grid, bf, s); break;
    case 14: launch_variant_tma<CL, MODE, 2, 5>(A, grid, bf, s); break;
    case 15: launch_variant_tma<CL, MODE, 0, 5>(A, grid, bf, s); break;
    case 16: launch_variant_tma<CL, MODE, 2, 4, 1>(A, grid, bf, s); break;
    default: launch_variant_tma<CL, MODE, 2, 4, 2>(A, grid, bf, s); break;
  }
}

// Number of sum-factorised variants the autotuner may choose from: 0..17
// pointwise with global records, 18..19 tile-local, 20..22 uniform box,
// 23..24 structured box grid (no records).
constexpr int kHex8Variants = 25;

// Whether a variant can run on the plan (tile tables; a uniform box mesh; a
// structured one, loss exponent 1).
bool hex8_variant_applies(const folgb_plan* p, int v) {
  if (v >= kHex8GridFirst) return p->box_grid != 0 && p->phys.loss_exponent == 1.0;
  if (v >= kHex8BoxFirst) return p->box_valid != 0;
  if (v >= kHex8TileFirst) return p->tiles > 0;
  return true;
}

// Launches the sum-factorised kernel when it applies (hex8, linear
// elasticity, 2x2x2 Gauss); returns 1 if it did, 0 otherwise.  The grid's
// block count is recomputed for the variant's block size; the caller's
// partial-sum buffers are sized for the smallest block (64 threads).
// Returns 2 when the tile-local kernel ran (the caller then finishes with
// launch_tile_boundary instead of the node gather) and 3 when the structured
// box grid kernel finished everything.  The residual path (MODE_RESIDUAL,
// records for the node gather) runs variant 11 in place of a tile-local
// variant and 21 in place of a grid variant; a grid variant that does not
// apply, or whose gradients go to host memory, runs 21, a box variant on a
// plan that is not a uniform box mesh 16.
static bool is_host_pointer(const void* q) {
  if (!q) return false;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, q) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

int launch_hex8_fast(const folgb_plan* p, const VecArgs& A, dim3 grid, int mode, cudaStream_t s) {
  if (p->etype != FOLGB_HEX8 || p->physics != FOLGB_ELASTIC || p->phys.num_gp != 2) return 0;
  int variant = p->hex8_variant;
  const bool bf = p->mat.has_bf != 0;
  if (variant >= kHex8GridFirst) {
    // gradients into host memory (pinned result buffers): the box kernel and
    // the gather write them over the host link faster than the grid kernel's
    // scattered node stores
    if (mode == MODE_LOSS && p->box_grid && A.exponent == 1.f && !is_host_pointer(A.out)) {
      trace_begin(KID_ELEM_LOSS, s);
      launch_box_grid(p, A, grid, variant == kHex8GridFirst ? 1 : 2, s);
      trace_end(KID_ELEM_LOSS, s);
      return 3;
    }
    variant = kHex8BoxFirst + 1;
  }
  if (variant >= kHex8BoxFirst && !p->box_valid) variant = 16;
  const bool box = variant >= kHex8BoxFirst;
  const bool tile = !box && variant >= kHex8TileFirst && p->tiles > 0;
  if (!box && variant >= kHex8TileFirst && (mode != MODE_LOSS || !tile)) variant = 11;
  trace_begin(mode == MODE_LOSS ? KID_ELEM_LOSS : KID_ELEM_RESIDUAL, s);
  if (box) {
    if (mode == MODE_LOSS) launch_box<MODE_LOSS>(p, A, grid, variant, s);
    else launch_box<MODE_RESIDUAL>(p, A, grid, variant, s);
  } else if (mode == MODE_LOSS && tile) {
    const bool pipe = variant == kHex8TileFirst;
    if (p->ctrl_layout == FOLGB_CONTROL_NODAL) launch_tile<FOLGB_CONTROL_NODAL>(p, A, (int)grid.y, bf, pipe, s);
    else launch_tile<FOLGB_CONTROL_ELEMENT>(p, A, (int)grid.y, bf, pipe, s);
  } else if (p->ctrl_layout == FOLGB_CONTROL_NODAL) {
    if (mode == MODE_LOSS) launch_cl_mode<FOLGB_CONTROL_NODAL, MODE_LOSS>(A, grid, bf, variant, s);
    else launch_cl_mode<FOLGB_CONTROL_NODAL, MODE_RESIDUAL>(A, grid, bf, variant, s);
  } else {
    if (mode == MODE_LOSS) launch_cl_mode<FOLGB_CONTROL_ELEMENT, MODE_LOSS>(A, grid, bf, variant, s);
    else launch_cl_mode<FOLGB_CONTROL_ELEMENT, MODE_RESIDUAL>(A, grid, bf, variant, s);
  }
  trace_end(mode == MODE_LOSS ? KID_ELEM_LOSS : KID_ELEM_RESIDUAL, s);
  return (mode == MODE_LOSS && tile) ? 2 : 1;
}

// Second launch of the tile-local path (the nodes shared by tiles), as a
// programmatic dependent of the tile kernel when pdl != 0.
int launch_tile_boundary(const folgb_plan* p, const VecArgs& A, int B, cudaStream_t s, int pdl) {
  const TileArgs T = tile_args(p);
  const int rescale = A.exponent != 1.f ? 1 : 0;
  int64_t work = rescale ? std::max<int64_t>(std::max<int64_t>(T.nb_nodes, T.ni_nodes), A.E) : T.nb_nodes;
  int blocks = (int)std::min<int64_t>((work + 255) / 256, (int64_t)num_sms() * 8);
  if (blocks < 1) blocks = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks, (unsigned)B);
  cfg.blockDim = dim3(256);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  trace_begin(KID_GATHER, s);
  if (p->ctrl_layout == FOLGB_CONTROL_NODAL) FOLGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_tile_boundary<true>, A, T, rescale));
  else FOLGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_tile_boundary<false>, A, T, rescale));
  trace_end(KID_GATHER, s);
  return FOLGB_OK;
}

int hex8_variant_count() { return kHex8Variants; }

}  // namespace folgb
