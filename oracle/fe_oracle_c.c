/* FP64 C restatement of folax's weighted-residual loss and its adjoint for the
 * thermal and small-strain elastic elements (quad4, hex8, tet4).
 *
 * TEST INFRASTRUCTURE ONLY: this file is a second oracle and the timed CPU
 * baseline.  It is compiled by oracle/build_c.py into oracle/_build/ and
 * loaded by oracle/c_oracle.py; only tests, the smoke check and the bench's
 * CPU legs use it.  tests/test_oracle_c.py pins it against the NumPy oracle
 * (oracle/fe_oracle.py), itself pinned against the reference's golden vectors.
 *
 * It follows the reference's algorithm step by step, including forming the
 * element matrix before the residual:
 *   element matrices   fol/loss_functions/thermal.py:28-49 (thermal),
 *                      fol/loss_functions/mechanical.py:98-117 (elastic);
 *   energy            e = u_e . stop_gradient(S_e u_e - F_e)
 *                      (thermal.py:47-49, mechanical.py:114-117);
 *   batch loss        sum over elements (fe_loss.py:166-176, 250-262);
 *   adjoint           dL/du = assembled residual, zero on Dirichlet dofs;
 *                      dL/dde = derivative of the energy value with S_e's
 *                      dependence on the control (what jax.grad gives).
 * Geometry and Gauss points: fol/geometries/quadrilateral_2d_4.py:16-70,
 * hexahedra_3d_8.py:16-114, tetrahedra_3d_4.py:16-60; the caller passes the
 * points and weights (oracle/fe_oracle.py:gauss_rule) so both oracles share
 * one point order.
 *
 * Neo-Hookean (AD variant) loss: energy = sum_gp w detJ psi(C) with
 *   3-D psi = mu/2 (J^-2/3 I1 - 3) - mu ln J + lam/2 ln^2 J
 *   (fol/constitutive_material_models/neo_hooke.py:129-135), 2-D
 *   psi = mu/2 (I1 - 2) - mu ln J + lam/2 ln^2 J (:178-181), mu and lam from the
 *   interpolated control (mechanical_neohooke_AD.py:264-267); its adjoint is
 *   the true energy gradient sum_gp w detJ (F S) dN/dx (what jax.grad of
 *   mechanical_neohooke_AD.py:279-293 gives) and dpsi/d(control).
 *
 * Element loop and nodal gather run under OpenMP; the nodal gather walks a
 * node -> (element, local node) incidence list in a fixed order and the total
 * is summed serially, so loss and adjoint do not depend on the thread count.
 *
 * Also here, for the solve checks: the BC-applied residual and Jacobian
 * assembled in FP64 into a given canonical CSR pattern
 * (fe_loss.py:191-207, 264-318; the row-only Dirichlet rule), and FP64
 * Jacobi-preconditioned CG on a CSR matrix (fe_solver.py:60-78 with CG, x0 = 0).
 * The assembly adds element entries with OpenMP atomics, so its values may
 * differ from run to run in the last bits of FP64 (far below every tolerance
 * they are used with).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { FEO_QUAD4 = 0, FEO_HEX8 = 1, FEO_TET4 = 2 };
enum { FEO_THERMAL = 0, FEO_ELASTIC = 1, FEO_NEOHOOKE = 2 };
enum { FEO_NODAL = 0, FEO_ELEMENT = 1 };

#define MAXN 8
#define MAXD 24

static const double kHexSigns[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                       {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
static const double kQuadSigns[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};

typedef struct {
  int et, ph, nen, dim, ndof, nv, ngp;
  const double* gp; /* ngp x 3 */
  const double* gw; /* ngp */
  double D[6][6];
  double bf[3];
  double beta, c;
  double mu1, lam1; /* neo-Hooke: mu, lambda for a unit control (mechanical_neohooke_AD.py:264-267) */
} Spec;

static void shape(const Spec* s, const double* xi, double* N, double dN[MAXN][3]) {
  if (s->et == FEO_TET4) {
    N[0] = 1.0 - xi[0] - xi[1] - xi[2];
    N[1] = xi[0];
    N[2] = xi[1];
    N[3] = xi[2];
    for (int a = 0; a < 4; ++a)
      for (int k = 0; k < 3; ++k) dN[a][k] = (a == 0) ? -1.0 : (a == k + 1 ? 1.0 : 0.0);
    return;
  }
  if (s->et == FEO_QUAD4) {
    for (int a = 0; a < 4; ++a) {
      const double fx = 1.0 + kQuadSigns[a][0] * xi[0], fy = 1.0 + kQuadSigns[a][1] * xi[1];
      N[a] = 0.25 * fx * fy;
      dN[a][0] = 0.25 * kQuadSigns[a][0] * fy;
      dN[a][1] = 0.25 * kQuadSigns[a][1] * fx;
      dN[a][2] = 0.0;
    }
    return;
  }
  for (int a = 0; a < 8; ++a) {
    const double f0 = 1.0 + kHexSigns[a][0] * xi[0], f1 = 1.0 + kHexSigns[a][1] * xi[1],
                 f2 = 1.0 + kHexSigns[a][2] * xi[2];
    N[a] = 0.125 * f0 * f1 * f2;
    dN[a][0] = 0.125 * kHexSigns[a][0] * f1 * f2;
    dN[a][1] = 0.125 * kHexSigns[a][1] * f0 * f2;
    dN[a][2] = 0.125 * kHexSigns[a][2] * f0 * f1;
  }
}

/* dN/dx = dN/dxi J^-1 with J[i][k] = sum_a X[a][i] dN_a/dxi_k (geometry.py:87-97). */
static double global_grads(const Spec* s, const double X[MAXN][3], double dN[MAXN][3], double G[MAXN][3]) {
  const int d = s->dim;
  double J[3][3] = {{0}};
  for (int a = 0; a < s->nen; ++a)
    for (int i = 0; i < d; ++i)
      for (int k = 0; k < d; ++k) J[i][k] += X[a][i] * dN[a][k];
  double det, Ji[3][3];
  if (d == 2) {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    Ji[0][0] = J[1][1] / det;
    Ji[0][1] = -J[0][1] / det;
    Ji[1][0] = -J[1][0] / det;
    Ji[1][1] = J[0][0] / det;
  } else {
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    Ji[0][0] = c00 / det;
    Ji[1][0] = c01 / det;
    Ji[2][0] = c02 / det;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  }
  for (int a = 0; a < s->nen; ++a)
    for (int j = 0; j < d; ++j) {
      double v = 0.0;
      for (int k = 0; k < d; ++k) v += dN[a][k] * Ji[k][j];
      G[a][j] = v;
    }
  return det;
}

/* Small-strain B in the reference's row order (mechanical.py:35-58):
 * 3-D rows xx, yy, zz, xy, yz, xz; 2-D rows xx, yy, xy. */
static void strain_B(const Spec* s, double G[MAXN][3], double B[6][MAXD]) {
  const int nd = s->nen * s->ndof;
  for (int v = 0; v < s->nv; ++v)
    for (int i = 0; i < nd; ++i) B[v][i] = 0.0;
  for (int a = 0; a < s->nen; ++a) {
    if (s->dim == 2) {
      B[0][2 * a] = G[a][0];
      B[1][2 * a + 1] = G[a][1];
      B[2][2 * a] = G[a][1];
      B[2][2 * a + 1] = G[a][0];
    } else {
      B[0][3 * a] = G[a][0];
      B[1][3 * a + 1] = G[a][1];
      B[2][3 * a + 2] = G[a][2];
      B[3][3 * a] = G[a][1];
      B[3][3 * a + 1] = G[a][0];
      B[4][3 * a + 1] = G[a][2];
      B[4][3 * a + 2] = G[a][1];
      B[5][3 * a] = G[a][2];
      B[5][3 * a + 2] = G[a][0];
    }
  }
}

/* One element: energy, residual re (nen*ndof), control gradient gde (nen).
 * Returns 0, or 1 when detJ <= 0 at some point. */
static inline __attribute__((always_inline)) int element(const Spec* s, const double X[MAXN][3],
                                                         const double* de, const double* ue, double* energy,
                                                         double* re, double* gde, double* Se_out) {
  const int nen = s->nen, nd = nen * s->ndof;
  double Se[MAXD][MAXD], Fe[MAXD];
  memset(Se, 0, sizeof(Se));
  memset(Fe, 0, sizeof(Fe));
  for (int a = 0; a < nen; ++a) gde[a] = 0.0;
  int bad = 0;
  for (int q = 0; q < s->ngp; ++q) {
    double N[MAXN], dN[MAXN][3], G[MAXN][3];
    shape(s, s->gp + 3 * q, N, dN);
    const double detJ = global_grads(s, X, dN, G);
    if (!(detJ > 0.0)) bad = 1;
    const double wd = s->gw[q] * detJ;
    double dgp = 0.0;
    for (int a = 0; a < nen; ++a) dgp += de[a] * N[a];
    if (s->ph == FEO_THERMAL) {
      double tgp = 0.0, gT[3] = {0, 0, 0};
      for (int a = 0; a < nen; ++a) {
        tgp += ue[a] * N[a];
        for (int j = 0; j < s->dim; ++j) gT[j] += ue[a] * G[a][j];
      }
      const double g = 1.0 + s->beta * pow(tgp, s->c);
      const double k = dgp * g;
      for (int a = 0; a < nen; ++a)
        for (int b = 0; b < nen; ++b) {
          double dd = 0.0;
          for (int j = 0; j < s->dim; ++j) dd += G[a][j] * G[b][j];
          Se[a][b] += wd * k * dd;
        }
      double gg = 0.0;
      for (int j = 0; j < s->dim; ++j) gg += gT[j] * gT[j];
      for (int a = 0; a < nen; ++a) gde[a] += wd * g * gg * N[a];
    } else {
      double B[6][MAXD], DB[6][MAXD], eps[6] = {0};
      strain_B(s, G, B);
      for (int v = 0; v < s->nv; ++v)
        for (int i = 0; i < nd; ++i) {
          double t = 0.0;
          for (int w = 0; w < s->nv; ++w) t += s->D[v][w] * B[w][i];
          DB[v][i] = t;
        }
      for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j) {
          double t = 0.0;
          for (int v = 0; v < s->nv; ++v) t += B[v][i] * DB[v][j];
          Se[i][j] += wd * dgp * t;
        }
      for (int a = 0; a < nen; ++a)
        for (int cc = 0; cc < s->ndof; ++cc) Fe[a * s->ndof + cc] += wd * N[a] * s->bf[cc];
      for (int v = 0; v < s->nv; ++v)
        for (int i = 0; i < nd; ++i) eps[v] += B[v][i] * ue[i];
      double eDe = 0.0;
      for (int v = 0; v < s->nv; ++v)
        for (int w = 0; w < s->nv; ++w) eDe += eps[v] * s->D[v][w] * eps[w];
      for (int a = 0; a < nen; ++a) gde[a] += wd * eDe * N[a];
    }
  }
  double en = 0.0;
  for (int i = 0; i < nd; ++i) {
    double t = -Fe[i];
    for (int j = 0; j < nd; ++j) t += Se[i][j] * ue[j];
    re[i] = t;
    en += ue[i] * t;
  }
  *energy = en;
  if (Se_out)
    for (int i = 0; i < nd; ++i)
      for (int j = 0; j < nd; ++j) Se_out[i * nd + j] = Se[i][j];
  return bad;
}

/* 3x3 / 2x2 determinant and inverse of a symmetric matrix C (d = 2 or 3). */
static double inv_sym(int d, const double C[3][3], double Ci[3][3]) {
  if (d == 2) {
    const double det = C[0][0] * C[1][1] - C[0][1] * C[1][0];
    Ci[0][0] = C[1][1] / det;
    Ci[1][1] = C[0][0] / det;
    Ci[0][1] = -C[0][1] / det;
    Ci[1][0] = -C[1][0] / det;
    return det;
  }
  const double c00 = C[1][1] * C[2][2] - C[1][2] * C[2][1];
  const double c01 = C[1][2] * C[2][0] - C[1][0] * C[2][2];
  const double c02 = C[1][0] * C[2][1] - C[1][1] * C[2][0];
  const double det = C[0][0] * c00 + C[0][1] * c01 + C[0][2] * c02;
  Ci[0][0] = c00 / det;
  Ci[1][0] = c01 / det;
  Ci[2][0] = c02 / det;
  Ci[0][1] = (C[0][2] * C[2][1] - C[0][1] * C[2][2]) / det;
  Ci[1][1] = (C[0][0] * C[2][2] - C[0][2] * C[2][0]) / det;
  Ci[2][1] = (C[0][1] * C[2][0] - C[0][0] * C[2][1]) / det;
  Ci[0][2] = (C[0][1] * C[1][2] - C[0][2] * C[1][1]) / det;
  Ci[1][2] = (C[0][2] * C[1][0] - C[0][0] * C[1][2]) / det;
  Ci[2][2] = (C[0][0] * C[1][1] - C[0][1] * C[1][0]) / det;
  return det;
}

/* Neo-Hookean (AD variant) element: energy sum_gp w detJ psi, re = the
 * energy gradient sum_gp w detJ (F S) dN/dx, gde[a] = d energy / d de[a]. */
static int element_nh(const Spec* s, const double X[MAXN][3], const double* de, const double* ue, double* energy,
                      double* re, double* gde) {
  const int nen = s->nen, d = s->dim, nd = nen * d;
  for (int i = 0; i < nd; ++i) re[i] = 0.0;
  for (int a = 0; a < nen; ++a) gde[a] = 0.0;
  double en = 0.0;
  int bad = 0;
  for (int q = 0; q < s->ngp; ++q) {
    double N[MAXN], dN[MAXN][3], G[MAXN][3];
    shape(s, s->gp + 3 * q, N, dN);
    const double detJ = global_grads(s, X, dN, G);
    if (!(detJ > 0.0)) bad = 1;
    const double wd = s->gw[q] * detJ;
    double egp = 0.0;
    for (int a = 0; a < nen; ++a) egp += de[a] * N[a];
    const double mu = s->mu1 * egp, lam = s->lam1 * egp;
    double F[3][3] = {{0}}, C[3][3] = {{0}}, Ci[3][3], S[3][3], P[3][3];
    for (int k = 0; k < d; ++k) {
      F[k][k] = 1.0;
      for (int j = 0; j < d; ++j)
        for (int a = 0; a < nen; ++a) F[k][j] += ue[a * d + k] * G[a][j];
    }
    for (int i = 0; i < d; ++i)
      for (int j = 0; j < d; ++j)
        for (int k = 0; k < d; ++k) C[i][j] += F[k][i] * F[k][j];
    const double detC = inv_sym(d, C, Ci);
    const double lnJ = 0.5 * log(detC);
    double I1 = 0.0;
    for (int i = 0; i < d; ++i) I1 += C[i][i];
    double psi, dpsi_dmu;
    if (d == 3) {
      const double aJ = exp(-2.0 / 3.0 * lnJ);
      psi = 0.5 * mu * (aJ * I1 - 3.0) - mu * lnJ + 0.5 * lam * lnJ * lnJ;
      dpsi_dmu = 0.5 * (aJ * I1 - 3.0) - lnJ;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          S[i][j] = mu * aJ * ((i == j ? 1.0 : 0.0) - I1 / 3.0 * Ci[i][j]) + (lam * lnJ - mu) * Ci[i][j];
    } else {
      psi = 0.5 * mu * (I1 - 2.0) - mu * lnJ + 0.5 * lam * lnJ * lnJ;
      dpsi_dmu = 0.5 * (I1 - 2.0) - lnJ;
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) S[i][j] = mu * ((i == j ? 1.0 : 0.0) - Ci[i][j]) + lam * lnJ * Ci[i][j];
    }
    const double dpsi_dlam = 0.5 * lnJ * lnJ;
    en += wd * psi;
    for (int k = 0; k < d; ++k)
      for (int j = 0; j < d; ++j) {
        double t = 0.0;
        for (int p = 0; p < d; ++p) t += F[k][p] * S[p][j];
        P[k][j] = t;
      }
    for (int a = 0; a < nen; ++a) {
      for (int k = 0; k < d; ++k) {
        double t = 0.0;
        for (int j = 0; j < d; ++j) t += P[k][j] * G[a][j];
        re[a * d + k] += wd * t;
      }
      gde[a] += wd * (dpsi_dmu * s->mu1 + dpsi_dlam * s->lam1) * N[a];
    }
  }
  *energy = en;
  return bad;
}

/* Copies of element() with the element type and physics as constants, so the
 * compiler sees fixed loop bounds (the same arithmetic, faster). */
#define FEO_SPECIALISE(NAME, ET, PH, NEN, DIM, NDOF, NV)                                                  \
  static int NAME(const Spec* s0, const double X[MAXN][3], const double* de, const double* ue, double* en, \
                  double* re, double* gde) {                                                              \
    Spec s = *s0;                                                                                         \
    s.et = ET;                                                                                            \
    s.ph = PH;                                                                                            \
    s.nen = NEN;                                                                                          \
    s.dim = DIM;                                                                                          \
    s.ndof = NDOF;                                                                                        \
    s.nv = NV;                                                                                            \
    return element(&s, X, de, ue, en, re, gde, NULL);                                                     \
  }
FEO_SPECIALISE(el_quad4_th, FEO_QUAD4, FEO_THERMAL, 4, 2, 1, 3)
FEO_SPECIALISE(el_hex8_th, FEO_HEX8, FEO_THERMAL, 8, 3, 1, 6)
FEO_SPECIALISE(el_tet4_th, FEO_TET4, FEO_THERMAL, 4, 3, 1, 6)
FEO_SPECIALISE(el_quad4_el, FEO_QUAD4, FEO_ELASTIC, 4, 2, 2, 3)
FEO_SPECIALISE(el_hex8_el, FEO_HEX8, FEO_ELASTIC, 8, 3, 3, 6)
FEO_SPECIALISE(el_tet4_el, FEO_TET4, FEO_ELASTIC, 4, 3, 3, 6)

#define FEO_SPECIALISE_NH(NAME, ET, NEN, DIM, NV)                                                         \
  static int NAME(const Spec* s0, const double X[MAXN][3], const double* de, const double* ue, double* en, \
                  double* re, double* gde) {                                                              \
    Spec s = *s0;                                                                                         \
    s.et = ET;                                                                                            \
    s.nen = NEN;                                                                                          \
    s.dim = DIM;                                                                                          \
    s.ndof = DIM;                                                                                         \
    s.nv = NV;                                                                                            \
    return element_nh(&s, X, de, ue, en, re, gde);                                                        \
  }
FEO_SPECIALISE_NH(el_quad4_nh, FEO_QUAD4, 4, 2, 3)
FEO_SPECIALISE_NH(el_hex8_nh, FEO_HEX8, 8, 3, 6)
FEO_SPECIALISE_NH(el_tet4_nh, FEO_TET4, 4, 3, 6)

typedef int (*ElementFn)(const Spec*, const double[MAXN][3], const double*, const double*, double*, double*,
                         double*);

static int make_spec(Spec* s, int et, int ph, int ngp, const double* gp, const double* gw, double young, double nu,
                     const double* bf, double beta, double c) {
  memset(s, 0, sizeof(*s));
  s->et = et;
  s->ph = ph;
  s->nen = et == FEO_HEX8 ? 8 : 4;
  s->dim = et == FEO_QUAD4 ? 2 : 3;
  if (et < 0 || et > 2 || ph < 0 || ph > 2 || ngp <= 0) return 1;
  s->ndof = ph == FEO_THERMAL ? 1 : s->dim;
  s->mu1 = 1.0 / (2.0 * (1.0 + nu));
  s->lam1 = nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  s->nv = s->dim == 2 ? 3 : 6;
  s->ngp = ngp;
  s->gp = gp;
  s->gw = gw;
  s->beta = beta;
  s->c = c;
  for (int i = 0; i < 3; ++i) s->bf[i] = bf ? bf[i] : 0.0;
  if (s->dim == 2) { /* plane stress (mechanical.py:60-61) */
    const double f = young / (1.0 - nu * nu);
    s->D[0][0] = s->D[1][1] = f;
    s->D[0][1] = s->D[1][0] = f * nu;
    s->D[2][2] = f * 0.5 * (1.0 - nu);
  } else { /* 3-D isotropic (mechanical.py:63-82) */
    const double c1 = young / ((1.0 + nu) * (1.0 - 2.0 * nu));
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) s->D[i][j] = c1 * nu;
    for (int i = 0; i < 3; ++i) s->D[i][i] = c1 * (1.0 - nu);
    for (int i = 3; i < 6; ++i) s->D[i][i] = c1 * 0.5 * (1.0 - 2.0 * nu);
  }
  return 0;
}

/* Loss and adjoint of one instance.
 *   conn (E x nen), xyz (N x 3), u: full dof vector (Dirichlet values applied),
 *   ctrl: N (nodal layout) or E (element layout) values,
 *   inc_ptr (N+1) / inc_slot: node -> slots e*nen+a in ascending order,
 *   dmask (ndof*N): 1 on Dirichlet dofs,
 *   rec (E*nen*ndof) and gde (E*nen): caller scratch.
 * Outputs: *total (sum of element energies), du (ndof*N) = assembled
 * residual with zeros on Dirichlet dofs, dctrl = d total / d ctrl.
 * Returns 0, 1 for bad arguments, 2 when an element has detJ <= 0. */
int feo_loss_adjoint(int et, int ph, int ngp, const double* gp, const double* gw, int layout, double young,
                     double nu, const double* bf, double beta, double c, int64_t E, const int64_t* conn, int64_t N,
                     const double* xyz, const int64_t* inc_ptr, const int64_t* inc_slot, const uint8_t* dmask,
                     const double* ctrl, const double* u, double* total, double* du, double* dctrl, double* rec,
                     double* gde, double* en, int nthreads) {
  Spec s;
  if (make_spec(&s, et, ph, ngp, gp, gw, young, nu, bf, beta, c)) return 1;
  const int nen = s.nen, ndof = s.ndof, nd = nen * ndof;
  static const ElementFn kFns[3][3] = {{el_quad4_th, el_hex8_th, el_tet4_th},
                                       {el_quad4_el, el_hex8_el, el_tet4_el},
                                       {el_quad4_nh, el_hex8_nh, el_tet4_nh}};
  const ElementFn fn = kFns[ph][et];
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t e = 0; e < E; ++e) {
    double X[MAXN][3], de[MAXN], ue[MAXD];
    for (int a = 0; a < nen; ++a) {
      const int64_t n = conn[e * nen + a];
      for (int k = 0; k < 3; ++k) X[a][k] = xyz[3 * n + k];
      de[a] = layout == FEO_ELEMENT ? ctrl[e] : ctrl[n];
      for (int cc = 0; cc < ndof; ++cc) ue[a * ndof + cc] = u[ndof * n + cc];
    }
    bad |= fn(&s, X, de, ue, en + e, rec + e * nd, gde + e * nen);
  }
  double t = 0.0;
  for (int64_t e = 0; e < E; ++e) t += en[e];
  *total = t;
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < N; ++n) {
    double acc[3] = {0, 0, 0}, ac = 0.0;
    for (int64_t k = inc_ptr[n]; k < inc_ptr[n + 1]; ++k) {
      const int64_t slot = inc_slot[k];
      for (int cc = 0; cc < ndof; ++cc) acc[cc] += rec[slot * ndof + cc];
      ac += gde[slot];
    }
    for (int cc = 0; cc < ndof; ++cc) du[ndof * n + cc] = dmask[ndof * n + cc] ? 0.0 : acc[cc];
    if (layout == FEO_NODAL) dctrl[n] = ac;
  }
  if (layout == FEO_ELEMENT) {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < E; ++e) {
      double a = 0.0;
      for (int k = 0; k < nen; ++k) a += gde[e * nen + k];
      dctrl[e] = a;
    }
  }
  return bad ? 2 : 0;
}

/* Position of column `col` in CSR row `row` (binary search of the sorted
 * column indices), or -1. */
static int64_t csr_find(const int32_t* rowptr, const int32_t* colind, int64_t row, int64_t col) {
  int64_t lo = rowptr[row], hi = rowptr[row + 1] - 1;
  while (lo <= hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (colind[mid] < col) lo = mid + 1;
    else if (colind[mid] > col) hi = mid - 1;
    else return mid;
  }
  return -1;
}

/* ComputeJacobianMatrixAndResidualVector (fe_loss.py:264-318) in FP64 for the
 * thermal and small-strain elastic elements: element residuals and matrices
 * with the row-only Dirichlet rule (fe_loss.py:191-207: a Dirichlet row keeps
 * only the element diagonal, its residual is zero), summed into the given
 * canonical CSR pattern (rowptr[rows+1], sorted colind).  dmask (ndof*N): 1
 * on Dirichlet dofs.  u: full dof vector.  Outputs residual (ndof*N) and
 * values (nnz).  Returns 0, 1 for bad arguments or an entry outside the
 * pattern, 2 when an element has detJ <= 0. */
int feo_assemble_csr(int et, int ph, int ngp, const double* gp, const double* gw, int layout, double young,
                     double nu, const double* bf, double beta, double c, int64_t E, const int64_t* conn, int64_t N,
                     const double* xyz, const uint8_t* dmask, const double* ctrl, const double* u,
                     const int32_t* rowptr, const int32_t* colind, double* residual, double* values, int nthreads) {
  Spec s;
  if (make_spec(&s, et, ph, ngp, gp, gw, young, nu, bf, beta, c) || ph == FEO_NEOHOOKE) return 1;
  const int nen = s.nen, ndof = s.ndof, nd = nen * ndof;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  const int64_t ndofs = ndof * N;
  memset(residual, 0, sizeof(double) * ndofs);
  memset(values, 0, sizeof(double) * rowptr[ndofs]);
  int bad = 0, miss = 0;
#pragma omp parallel for schedule(static) reduction(| : bad, miss)
  for (int64_t e = 0; e < E; ++e) {
    double X[MAXN][3], de[MAXN], ue[MAXD], re[MAXD], gde[MAXN], Se[MAXD * MAXD], en;
    int64_t dof[MAXD];
    for (int a = 0; a < nen; ++a) {
      const int64_t n = conn[e * nen + a];
      for (int k = 0; k < 3; ++k) X[a][k] = xyz[3 * n + k];
      de[a] = layout == FEO_ELEMENT ? ctrl[e] : ctrl[n];
      for (int cc = 0; cc < ndof; ++cc) {
        dof[a * ndof + cc] = ndof * n + cc;
        ue[a * ndof + cc] = u[ndof * n + cc];
      }
    }
    bad |= element(&s, X, de, ue, &en, re, gde, Se);
    for (int i = 0; i < nd; ++i) {
      const int64_t r = dof[i];
      const int keep_row = !dmask[r];
      if (keep_row) {
#pragma omp atomic
        residual[r] += re[i];
      }
      for (int j = 0; j < nd; ++j) {
        double v = Se[i * nd + j];
        if (!keep_row) v = (i == j) ? v : 0.0;
        if (v == 0.0 && !(i == j)) continue;
        const int64_t pos = csr_find(rowptr, colind, r, dof[j]);
        if (pos < 0) {
          miss = 1;
          continue;
        }
#pragma omp atomic
        values[pos] += v;
      }
    }
  }
  if (miss) return 1;
  return bad ? 2 : 0;
}

/* FP64 Jacobi-preconditioned CG with x0 = 0 on a CSR matrix (rows x rows,
 * int32 pattern, double values): stops when the true residual
 * ||b - A x|| <= rtol ||b|| (the recurrence residual is replaced by b - A x
 * every 50 iterations and whenever it reaches the tolerance) or at maxiter.
 * Writes x; returns the iteration count, -1 for bad arguments. */
int64_t feo_pcg(int64_t rows, const int32_t* rowptr, const int32_t* colind, const double* values, const double* b,
                double* x, double rtol, int64_t maxiter, double* rel_residual, double* work, int nthreads) {
  if (rows <= 0 || !rowptr || !colind || !values || !b || !x || !work) return -1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  double *r = work, *z = work + rows, *p = work + 2 * rows, *q = work + 3 * rows, *dinv = work + 4 * rows;
  double bn = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : bn)
  for (int64_t i = 0; i < rows; ++i) {
    double d = 0.0;
    for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if (colind[k] == i) d = values[k];
    dinv[i] = d != 0.0 ? 1.0 / d : 0.0;
    x[i] = 0.0;
    r[i] = b[i];
    z[i] = dinv[i] * r[i];
    p[i] = z[i];
    bn += b[i] * b[i];
  }
  bn = sqrt(bn);
  if (rel_residual) *rel_residual = 0.0;
  if (bn == 0.0) return 0;
  double rz = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rz)
  for (int64_t i = 0; i < rows; ++i) rz += r[i] * z[i];
  int64_t it = 0;
  double rn = bn;
  while (it < maxiter) {
    ++it;
    double pq = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : pq)
    for (int64_t i = 0; i < rows; ++i) {
      double t = 0.0;
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) t += values[k] * p[colind[k]];
      q[i] = t;
      pq += p[i] * t;
    }
    const double alpha = rz / pq;
    double rr = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rr)
    for (int64_t i = 0; i < rows; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      rr += r[i] * r[i];
    }
    /* the true residual b - A x every 50 iterations and before stopping */
    if ((it % 50) == 0 || sqrt(rr) <= rtol * bn) {
      rr = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rr)
      for (int64_t i = 0; i < rows; ++i) {
        double t = b[i];
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) t -= values[k] * x[colind[k]];
        r[i] = t;
        rr += t * t;
      }
    }
    rn = sqrt(rr);
    if (rn <= rtol * bn) break;
    double rz_new = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rz_new)
    for (int64_t i = 0; i < rows; ++i) {
      z[i] = dinv[i] * r[i];
      rz_new += r[i] * z[i];
    }
    const double beta_ = rz_new / rz;
    rz = rz_new;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < rows; ++i) p[i] = z[i] + beta_ * p[i];
  }
  if (rel_residual) *rel_residual = rn / bn;
  return it;
}

int feo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
