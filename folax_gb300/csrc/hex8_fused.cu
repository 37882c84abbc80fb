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

template <int CL, int MODE>
__global__ void __launch_bounds__(256) k_hex8_elastic(const VecArgs A) {
  __shared__ float red[32];
  const int b = blockIdx.y;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float energy = 0.f;
  int bad = 0;
  if (e < A.E) {
    constexpr int LEX[8] = {0, 1, 3, 2, 4, 5, 7, 6};  // lex position -> node
    int nodes[8];
    load_nodes<8>(A.conn, e, nodes);
    const float* dofs = A.dofs + (int64_t)b * A.dofs_stride;
    const float* ctrl = A.ctrl + (int64_t)b * A.ctrl_stride;
    float X[3][8], U[3][8], de[8];
#pragma unroll
    for (int L = 0; L < 8; ++L) {
      const int n = nodes[LEX[L]];
      const float4 x = __ldg(A.xyz4 + n);
      X[0][L] = x.x;
      X[1][L] = x.y;
      X[2][L] = x.z;
      const unsigned m = A.apply_dirichlet ? __ldg(A.dmask + n) : 0u;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int64_t d = 3 * (int64_t)n + c;
        U[c][L] = ((m >> c) & 1u) ? __ldg(A.dval + d) : __ldg(dofs + d);
      }
      if (CL == FOLGB_CONTROL_NODAL) de[L] = __ldg(ctrl + n);
    }
    float egp[8];
    if (CL == FOLGB_CONTROL_NODAL) {
#pragma unroll
      for (int L = 0; L < 8; ++L) egp[L] = de[L];
      interp8(egp);
    } else {
      const float ev = __ldg(ctrl + e);
#pragma unroll
      for (int q = 0; q < 8; ++q) egp[q] = ev;
    }
    // reference derivatives of the geometry and of the displacement
    Deriv12 DX[3], DU[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      wht8(X[i]);
      deriv12(X[i], DX[i]);
      wht8(U[i]);
      deriv12(U[i], DU[i]);
    }
    // per-direction adjoint accumulators S[i][dir][4]
    float S[3][3][4];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int t = 0; t < 4; ++t) S[i][k][t] = 0.f;
    float wsed[8], wdet[8];
    const MatConst& mt = A.mat;
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
      wdet[q] = wd;
      float H[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) H[i][j] = Gm[i][0] * Ji[0][j] + Gm[i][1] * Ji[1][j] + Gm[i][2] * Ji[2][j];
      const float tr = H[0][0] + H[1][1] + H[2][2];
      const float g01 = H[0][1] + H[1][0], g12 = H[1][2] + H[2][1], g02 = H[0][2] + H[2][0];
      const float sed = mt.lam * tr * tr + 2.f * mt.mu * (H[0][0] * H[0][0] + H[1][1] * H[1][1] + H[2][2] * H[2][2]) +
                        mt.mu * (g01 * g01 + g12 * g12 + g02 * g02);
      const float ew = egp[q] * wd;
      energy = fmaf(ew, sed, energy);
      wsed[q] = wd * sed;
      // w detJ sigma
      const float lt = ew * mt.lam * tr, tm = 2.f * ew * mt.mu, sm = ew * mt.mu;
      float sg[3][3];
      sg[0][0] = fmaf(tm, H[0][0], lt);
      sg[1][1] = fmaf(tm, H[1][1], lt);
      sg[2][2] = fmaf(tm, H[2][2], lt);
      sg[0][1] = sg[1][0] = sm * g01;
      sg[1][2] = sg[2][1] = sm * g12;
      sg[0][2] = sg[2][0] = sm * g02;
      // T[i][k] = sum_j sg[i][j] Ji[k][j]; scatter into the direction sums
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float t0 = sg[i][0] * Ji[0][0] + sg[i][1] * Ji[0][1] + sg[i][2] * Ji[0][2];
        const float t1 = sg[i][0] * Ji[1][0] + sg[i][1] * Ji[1][1] + sg[i][2] * Ji[1][2];
        const float t2 = sg[i][0] * Ji[2][0] + sg[i][1] * Ji[2][1] + sg[i][2] * Ji[2][2];
        S[i][0][ix] += t0;
        S[i][1][iy] += t1;
        S[i][2][iz] += t2;
      }
    }
    // adjoint: per component, dual Hadamard coefficients then the transposed transform
    float g[8][3];
    const float s = 0.125f, sg_ = 0.125f * kG, sg2 = 0.125f * kG2;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      float d[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) d[k] = 0.f;
      float A1 = 0.f, B1 = 0.f, C1 = 0.f, D1 = 0.f;
      butterfly4_t(S[i][0], A1, B1, C1, D1);  // xi: (1, xi eta, xi zeta, xi eta zeta)
      d[1] += s * A1;
      d[3] += sg_ * B1;
      d[5] += sg_ * C1;
      d[7] += sg2 * D1;
      float A2 = 0.f, B2 = 0.f, C2 = 0.f, D2 = 0.f;
      butterfly4_t(S[i][1], A2, B2, C2, D2);  // eta: (eta, xi eta, eta zeta, xi eta zeta)
      d[2] += s * A2;
      d[3] += sg_ * B2;
      d[6] += sg_ * C2;
      d[7] += sg2 * D2;
      float A3 = 0.f, B3 = 0.f, C3 = 0.f, D3 = 0.f;
      butterfly4_t(S[i][2], A3, B3, C3, D3);  // zeta: (zeta, xi zeta, eta zeta, xi eta zeta)
      d[4] += s * A3;
      d[5] += sg_ * B3;
      d[6] += sg_ * C3;
      d[7] += sg2 * D3;
      wht8_t(d);
#pragma unroll
      for (int L = 0; L < 8; ++L) g[L][i] = d[L];
    }
    if (mt.has_bf) {
      float W[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) W[q] = wdet[q];
      interp8(W);
#pragma unroll
      for (int L = 0; L < 8; ++L)
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const float f = W[L] * mt.bf[i];
          g[L][i] -= f;
          // u was transformed in place: recompute the nodal value from the dofs
          const int n = nodes[LEX[L]];
          const unsigned m = A.apply_dirichlet ? __ldg(A.dmask + n) : 0u;
          const int64_t dd = 3 * (int64_t)n + i;
          const float uv = ((m >> i) & 1u) ? __ldg(A.dval + dd) : __ldg(dofs + dd);
          energy = fmaf(-f, uv, energy);
        }
    }
    if (!isfinite(energy)) bad |= 2;
    // element vector in node order, 16-byte stores
    float out[24];
#pragma unroll
    for (int L = 0; L < 8; ++L)
#pragma unroll
      for (int i = 0; i < 3; ++i) out[3 * LEX[L] + i] = g[L][i];
    float4* gout = reinterpret_cast<float4*>(A.g + ((int64_t)b * A.E + e) * 24);
#pragma unroll
    for (int k = 0; k < 6; ++k) gout[k] = make_float4(out[4 * k], out[4 * k + 1], out[4 * k + 2], out[4 * k + 3]);
    if (MODE == MODE_LOSS) {
      if (CL == FOLGB_CONTROL_NODAL) {
        interp8(wsed);
        float gn[8];
#pragma unroll
        for (int L = 0; L < 8; ++L) gn[LEX[L]] = wsed[L];
        float4* go = reinterpret_cast<float4*>(A.gde + ((int64_t)b * A.E + e) * 8);
        go[0] = make_float4(gn[0], gn[1], gn[2], gn[3]);
        go[1] = make_float4(gn[4], gn[5], gn[6], gn[7]);
      } else if (A.dctrl_elem) {
        float sum = 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) sum += wsed[q];
        A.dctrl_elem[(int64_t)b * A.E + e] = (A.exponent == 1.f) ? sum * A.inv_batch : sum;
      }
    }
  }
  report_bad(bad, A.status);
  if (MODE == MODE_LOSS) {
    float be = block_sum(energy, red);
    finish_loss(be, A, b, red);
  }
}

// Launches the sum-factorised kernel when it applies (hex8, linear
// elasticity, 2x2x2 Gauss); returns 1 if it did, 0 otherwise.
int launch_hex8_fast(const folgb_plan* p, const VecArgs& A, dim3 grid, int mode, cudaStream_t s) {
  if (p->etype != FOLGB_HEX8 || p->physics != FOLGB_ELASTIC || p->phys.num_gp != 2) return 0;
  trace_begin(mode == MODE_LOSS ? KID_ELEM_LOSS : KID_ELEM_RESIDUAL, s);
  if (p->ctrl_layout == FOLGB_CONTROL_NODAL) {
    if (mode == MODE_LOSS) k_hex8_elastic<FOLGB_CONTROL_NODAL, MODE_LOSS><<<grid, 256, 0, s>>>(A);
    else k_hex8_elastic<FOLGB_CONTROL_NODAL, MODE_RESIDUAL><<<grid, 256, 0, s>>>(A);
  } else {
    if (mode == MODE_LOSS) k_hex8_elastic<FOLGB_CONTROL_ELEMENT, MODE_LOSS><<<grid, 256, 0, s>>>(A);
    else k_hex8_elastic<FOLGB_CONTROL_ELEMENT, MODE_RESIDUAL><<<grid, 256, 0, s>>>(A);
  }
  trace_end(mode == MODE_LOSS ? KID_ELEM_LOSS : KID_ELEM_RESIDUAL, s);
  return 1;
}

}  // namespace folgb
