// Uniform box meshes: every hexahedron is the same axis-aligned box.
//
// The reference evaluates each element's energy and residual point by point
// (fol/loss_functions/mechanical.py:98-117, 2x2x2 Gauss rule of
// hexahedra_3d_8.py:22-33).  For linear elasticity the element energy is a
// quadratic form of the 24 nodal displacements, e(u) = E_e u.K u, with
// residual K u, and on a mesh whose elements are all translates of one box K
// is the same for every element.  In the Walsh-Hadamard basis of the nodal
// values (per displacement component, the transform the sum-factorised
// kernels already use) K is block diagonal: the reflections of the box
// through its mid-planes map the box, the Gauss rule and an isotropic
// material onto themselves, and a mode (component c, Hadamard index b) has
// the reflection parity p = b xor (1 << c); modes of different parity do not
// couple.  That leaves eight 3 x 3 blocks, one per parity, with the modes
// (0, p^1), (1, p^2), (2, p^4).  A box element then costs two 8-point
// transforms per component, 72 multiply-adds for the blocks and 24 for the
// energy, against about 1,300 instructions for the pointwise evaluation.
//
// The plan builds the blocks once, in FP64, from the same bilinear form the
// pointwise kernels evaluate (sed = lambda tr(H)^2 + 2 mu sum_i H_ii^2 +
// mu sum_{i<j} (H_ij + H_ji)^2 at each Gauss point, weight detJ), and keeps
// them only when every element's coordinates (the plan's fp32 values) give
// exactly the same diagonal Jacobian and no bilinear or trilinear term, and
// the off-block entries vanish.
#include <cmath>
#include <vector>

#include "folgb_internal.cuh"

namespace folgb {

namespace {

constexpr int kLexNode[8] = {0, 1, 3, 2, 4, 5, 7, 6};  // lexicographic position -> reference local node

// h[b] = sum_L f[L] prod_d s(L_d)^(b_d), s(0) = -1, s(1) = +1 (the kernels' wht8)
void wht8_host(double (&f)[8]) {
  for (int st = 1; st < 8; st <<= 1)
    for (int L = 0; L < 8; ++L)
      if (!(L & st)) {
        const double a = f[L], b = f[L + st];
        f[L] = a + b;
        f[L + st] = b - a;
      }
}

double hsign(int b, int L) {
  double s = 1.0;
  for (int d = 0; d < 3; ++d)
    if (((b >> d) & 1) && !((L >> d) & 1)) s = -s;
  return s;
}

}  // namespace

// The 24 x 24 element matrix of one box in the Hadamard basis, FP64:
// khat[(c, b)][(c', b')] (index 8 c + b) = (1/64) sum_{L, L'} H_bL K_(c,L)(c',L') H_b'L'
// with u.K u = sum_q detJ sed(H_q(u)).  J is the box's Jacobian (rows:
// coordinates, columns: reference directions).
void box_hadamard_stiffness(const double (&J)[3][3], double lam, double mu, double (&khat)[24][24]) {
  // inverse and determinant of J
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  double Ji[3][3];
  Ji[0][0] = c00 / det;
  Ji[1][0] = c01 / det;
  Ji[2][0] = c02 / det;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  const double g = 1.0 / std::sqrt(3.0);
  double K[24][24] = {};
  for (int q = 0; q < 8; ++q) {
    double xi[3];
    for (int d = 0; d < 3; ++d) xi[d] = ((q >> d) & 1) ? g : -g;
    // physical gradient row of each lexicographic node's shape function
    double grad[8][3];
    for (int L = 0; L < 8; ++L) {
      double dref[3];
      for (int k = 0; k < 3; ++k) {
        double v = 0.5 * (((L >> k) & 1) ? 1.0 : -1.0);
        for (int d = 0; d < 3; ++d)
          if (d != k) v *= 0.5 * (1.0 + (((L >> d) & 1) ? 1.0 : -1.0) * xi[d]);
        dref[k] = v;
      }
      for (int j = 0; j < 3; ++j) grad[L][j] = dref[0] * Ji[0][j] + dref[1] * Ji[1][j] + dref[2] * Ji[2][j];
    }
    // unit dof (c, L): H = e_c grad_L^T (only row c)
    for (int c = 0; c < 3; ++c)
      for (int L = 0; L < 8; ++L)
        for (int c2 = 0; c2 < 3; ++c2)
          for (int L2 = 0; L2 < 8; ++L2) {
            double Ha[3][3] = {}, Hb[3][3] = {};
            for (int j = 0; j < 3; ++j) {
              Ha[c][j] = grad[L][j];
              Hb[c2][j] = grad[L2][j];
            }
            const double tra = Ha[0][0] + Ha[1][1] + Ha[2][2], trb = Hb[0][0] + Hb[1][1] + Hb[2][2];
            double v = lam * tra * trb;
            for (int i = 0; i < 3; ++i) v += 2.0 * mu * Ha[i][i] * Hb[i][i];
            for (int i = 0; i < 3; ++i)
              for (int j = i + 1; j < 3; ++j) v += mu * (Ha[i][j] + Ha[j][i]) * (Hb[i][j] + Hb[j][i]);
            K[8 * c + L][8 * c2 + L2] += det * v;  // Gauss weight 1
          }
  }
  for (int c = 0; c < 3; ++c)
    for (int b = 0; b < 8; ++b)
      for (int c2 = 0; c2 < 3; ++c2)
        for (int b2 = 0; b2 < 8; ++b2) {
          double v = 0.0;
          for (int L = 0; L < 8; ++L)
            for (int L2 = 0; L2 < 8; ++L2) v += hsign(b, L) * K[8 * c + L][8 * c2 + L2] * hsign(b2, L2);
          khat[8 * c + b][8 * c2 + b2] = v / 64.0;
        }
}

int build_uniform_box(folgb_plan* p, const std::vector<float4>& x4, const std::vector<int>& conn,
                      const std::vector<unsigned char>& dmask) {
  p->box_valid = 0;
  if (p->etype != FOLGB_HEX8 || p->physics != FOLGB_ELASTIC || p->phys.num_gp != 2 ||
      p->ctrl_layout != FOLGB_CONTROL_ELEMENT || p->mat.has_bf || p->E <= 0)
    return FOLGB_OK;
  double J0[3][3] = {};
  for (int64_t e = 0; e < p->E; ++e) {
    double h[3][8];
    for (int L = 0; L < 8; ++L) {
      const float4 x = x4[conn[(size_t)e * 8 + kLexNode[L]]];
      h[0][L] = x.x;
      h[1][L] = x.y;
      h[2][L] = x.z;
    }
    for (int i = 0; i < 3; ++i) {
      wht8_host(h[i]);  // exact: sums of 8 fp32 values in fp64
      if (h[i][3] != 0.0 || h[i][5] != 0.0 || h[i][6] != 0.0 || h[i][7] != 0.0) return FOLGB_OK;
    }
    for (int i = 0; i < 3; ++i) {
      const double Ji[3] = {0.125 * h[i][1], 0.125 * h[i][2], 0.125 * h[i][4]};
      for (int k = 0; k < 3; ++k) {
        if (e == 0) J0[i][k] = Ji[k];
        else if (Ji[k] != J0[i][k]) return FOLGB_OK;
      }
    }
  }
  // an axis-aligned box with positive volume
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k)
      if (i != k && J0[i][k] != 0.0) return FOLGB_OK;
  if (!(J0[0][0] > 0.0 && J0[1][1] > 0.0 && J0[2][2] > 0.0)) return FOLGB_OK;
  double khat[24][24];
  box_hadamard_stiffness(J0, (double)p->mat.lam, (double)p->mat.mu, khat);
  double mx = 0.0;
  for (int a = 0; a < 24; ++a)
    for (int b = 0; b < 24; ++b) mx = std::fmax(mx, std::fabs(khat[a][b]));
  if (!(mx > 0.0) || !std::isfinite(mx)) return FOLGB_OK;
  const double tiny = 1e-13 * mx;
  for (int a = 0; a < 24; ++a)
    for (int b = 0; b < 24; ++b) {
      const int pa = (a & 7) ^ (1 << (a >> 3)), pb = (b & 7) ^ (1 << (b >> 3));
      if (pa != pb && std::fabs(khat[a][b]) > tiny) return FOLGB_OK;
    }
  for (int par = 0; par < 8; ++par)
    for (int c = 0; c < 3; ++c)
      for (int c2 = 0; c2 < 3; ++c2) {
        const double v = khat[8 * c + (par ^ (1 << c))][8 * c2 + (par ^ (1 << c2))];
        p->box_k.k[par][c][c2] = std::fabs(v) > tiny ? (float)v : 0.f;  // rigid translations: exact zeros
      }
  p->box_valid = 1;
  // the box mesh numbering: node (i, j, k) = i + NX (j + NY k), element
  // (i, j, k) = i + nx (j + ny k), local nodes in the reference order
  const int64_t NX = (int64_t)conn[3] - conn[0], NXY = (int64_t)conn[4] - conn[0];
  if (conn[0] != 0 || NX < 2 || NXY < 2 * NX || NXY % NX) return FOLGB_OK;
  const int64_t nx = NX - 1, ny = NXY / NX - 1;
  if (p->E % (nx * ny)) return FOLGB_OK;
  const int64_t nz = p->E / (nx * ny);
  // 32-bit dof offsets in the grid kernel: fewer than 2^31 dofs
  if (p->N != NXY * (nz + 1) || 3 * p->N >= ((int64_t)1 << 31)) return FOLGB_OK;
  constexpr int dx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, dy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, dz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  for (int64_t e = 0; e < p->E; ++e) {
    const int64_t i = e % nx, j = (e / nx) % ny, k = e / (nx * ny);
    for (int a = 0; a < 8; ++a)
      if (conn[(size_t)e * 8 + a] != (i + dx[a]) + NX * ((j + dy[a]) + (ny + 1) * (k + dz[a]))) return FOLGB_OK;
  }
  // node layers with a Dirichlet dof (the grid kernel reads masks only there)
  std::vector<unsigned char> layer_bc((size_t)nz + 1, 0);
  for (int64_t n = 0; n < p->N; ++n)
    if (dmask[(size_t)n]) layer_bc[(size_t)(n / NXY)] = 1;
  FOLGB_CUDA_TRY(cudaMalloc((void**)&p->d_box_layer_bc, layer_bc.size()));
  FOLGB_CUDA_TRY(cudaMemcpy(p->d_box_layer_bc, layer_bc.data(), layer_bc.size(), cudaMemcpyHostToDevice));
  p->box_grid = 1;
  p->box_nx = (int)nx;
  p->box_ny = (int)ny;
  p->box_nz = (int)nz;
  return FOLGB_OK;
}

}  // namespace folgb
