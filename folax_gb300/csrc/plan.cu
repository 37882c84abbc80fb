// Per-mesh tables: built once on the host (deterministic, single pass
// counting sorts) and uploaded to the device.  This is the GB300 analogue of
// FiniteElementLoss.Initialize (fol/loss_functions/fe_loss.py:57-122) plus the
// index work the reference redoes inside every jit call (element Jacobian
// indices, fe_loss.py:178-184, and the BCOO -> CSR conversion of
// fol/solvers/fe_solver.py:71-72).
#include <atomic>
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <numeric>

#include "folgb_internal.cuh"

using namespace folgb;

namespace folgb {

// SM count of the current device, cached per device ordinal (racing threads
// store the same value).
int num_sms() {
  constexpr int kDevs = 64;
  static std::atomic<int> cache[kDevs];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevs) dev = 0;
  int sms = cache[dev].load(std::memory_order_relaxed);
  if (sms == 0) {
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
    cache[dev].store(sms, std::memory_order_relaxed);
  }
  return sms;
}

static void gauss_1d(int order, std::vector<double>& x, std::vector<double>& w) {
  if (order == 1) {
    x = {0.0};
    w = {2.0};
  } else if (order == 2) {
    double g = 1.0 / std::sqrt(3.0);
    x = {-g, g};
    w = {1.0, 1.0};
  } else {
    double a = std::sqrt(3.0 / 5.0);
    x = {-a, 0.0, a};
    w = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
  }
}

// Gauss rules in the reference's point order (fol/geometries/quadrilateral_2d_4.py:16-45,
// hexahedra_3d_8.py:16-70, tetrahedra_3d_4.py:16-48).
static bool build_gp_table(int etype, int order, GPTable& t) {
  static const double hs[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                  {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  static const double qs[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
  if (order < 1 || order > 3) return false;
  std::vector<std::array<double, 3>> pts;
  std::vector<double> wts;
  if (etype == FOLGB_TET4) {
    if (order == 1) {
      pts.push_back({0.25, 0.25, 0.25});
      wts.push_back(1.0 / 6.0);
    } else if (order == 2) {
      double a = 0.58541020, b = 0.13819660;
      pts = {{a, b, b}, {b, a, b}, {b, b, a}, {b, b, b}};
      wts.assign(4, 1.0 / 24.0);
    } else {
      const double orb[2][3] = {{0.015835909865720057993, 0.32805469671142664734, 0.02308799441864369039},
                                {0.67914317820120795168, 0.10695227393293068277, 0.01857867224802297628}};
      for (auto& o : orb) {
        pts.push_back({o[0], o[1], o[1]});
        pts.push_back({o[1], o[0], o[1]});
        pts.push_back({o[1], o[1], o[0]});
        pts.push_back({o[1], o[1], o[1]});
        for (int k = 0; k < 4; ++k) wts.push_back(o[2]);
      }
    }
  } else {
    int dim = etype == FOLGB_QUAD4 ? 2 : 3;
    std::vector<double> x, w;
    gauss_1d(order, x, w);
    if (order == 2) {
      double g = x[1];
      if (dim == 2)
        for (auto& s : qs) pts.push_back({s[0] * g, s[1] * g, 0.0});
      else
        for (auto& s : hs) pts.push_back({s[0] * g, s[1] * g, s[2] * g});
      wts.assign(pts.size(), 1.0);
    } else {
      int n = (int)x.size();
      int nz = dim == 3 ? n : 1;
      for (int k = 0; k < nz; ++k)
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i) {
            pts.push_back({x[i], x[j], dim == 3 ? x[k] : 0.0});
            wts.push_back(w[i] * w[j] * (dim == 3 ? w[k] : 1.0));
          }
    }
  }
  std::memset(&t, 0, sizeof(t));
  t.npts = (int)pts.size();
  for (int q = 0; q < t.npts; ++q) {
    const double* p = pts[q].data();
    t.w[q] = (float)wts[q];
    if (etype == FOLGB_TET4) {
      double N[4] = {1.0 - p[0] - p[1] - p[2], p[0], p[1], p[2]};
      double dN[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
      for (int a = 0; a < 4; ++a) {
        t.N[q][a] = (float)N[a];
        for (int k = 0; k < 3; ++k) t.dN[q][a][k] = (float)dN[a][k];
      }
    } else if (etype == FOLGB_QUAD4) {
      for (int a = 0; a < 4; ++a) {
        double sx = qs[a][0], sy = qs[a][1];
        t.N[q][a] = (float)(0.25 * (1 + sx * p[0]) * (1 + sy * p[1]));
        t.dN[q][a][0] = (float)(0.25 * sx * (1 + sy * p[1]));
        t.dN[q][a][1] = (float)(0.25 * sy * (1 + sx * p[0]));
        t.dN[q][a][2] = 0.f;
      }
    } else {
      for (int a = 0; a < 8; ++a) {
        double f0 = 1 + hs[a][0] * p[0], f1 = 1 + hs[a][1] * p[1], f2 = 1 + hs[a][2] * p[2];
        t.N[q][a] = (float)(0.125 * f0 * f1 * f2);
        t.dN[q][a][0] = (float)(0.125 * hs[a][0] * f1 * f2);
        t.dN[q][a][1] = (float)(0.125 * hs[a][1] * f0 * f2);
        t.dN[q][a][2] = (float)(0.125 * hs[a][2] * f0 * f1);
      }
    }
  }
  return true;
}

template <class T>
static int upload(T** dst, const T* src, size_t n) {
  if (n == 0) n = 1;
  FOLGB_CUDA_TRY(cudaMalloc((void**)dst, n * sizeof(T)));
  if (src) FOLGB_CUDA_TRY(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return FOLGB_OK;
}

int fill_material(const folgb_physics& p, int dim, MatConst& m) {
  double nu = p.poisson_ratio, E = p.young_modulus;
  if (!(nu > -1.0 && nu < 0.5)) return FOLGB_ERR_INVALID_ARGUMENT;
  if (dim == 3) {
    m.lam = (float)(E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)));
    m.mu = (float)(E / (2.0 * (1.0 + nu)));
  } else {  // plane stress (fol/loss_functions/mechanical.py:60-61)
    m.lam = (float)(E * nu / (1.0 - nu * nu));
    m.mu = (float)(E / (2.0 * (1.0 + nu)));
  }
  m.mu_f = (float)(1.0 / (2.0 * (1.0 + nu)));
  m.lam_f = (float)(nu / ((1.0 + nu) * (1.0 - 2.0 * nu)));
  // bulk modulus per unit Young's modulus, the 3-D one in 2-D as well
  // (mechanical_neohooke.py:254)
  m.kap_f = (float)(1.0 / (3.0 * (1.0 - 2.0 * nu)));
  m.beta = (float)p.beta;
  m.c = (float)p.c;
  for (int i = 0; i < 3; ++i) m.bf[i] = (float)p.body_force[i];
  m.has_bf = (p.body_force[0] != 0.0 || p.body_force[1] != 0.0 || p.body_force[2] != 0.0) ? 1 : 0;
  m.shear_ref = p.shear_mode == FOLGB_SHEAR_REFERENCE ? 1 : 0;
  m.rho_cp = (float)p.rho_cp;
  m.dt = (float)p.time_step;
  m.mbeta = (float)p.material_beta;
  return FOLGB_OK;
}

// Node -> incident element slots, ascending element id (a stable counting sort).
void build_incidence(const std::vector<int>& conn, int64_t E, int nen, int64_t N, std::vector<int>& ptr,
                     std::vector<int>& slot) {
  ptr.assign(N + 1, 0);
  for (int64_t s = 0; s < E * nen; ++s) ptr[conn[s] + 1]++;
  for (int64_t n = 0; n < N; ++n) ptr[n + 1] += ptr[n];
  slot.assign(E * nen, 0);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int64_t s = 0; s < E * nen; ++s) slot[fill[conn[s]]++] = (int)s;
}

static int build_csr_tables(folgb_plan* p, const std::vector<int>& conn, const std::vector<int>& inc_ptr,
                            const std::vector<int>& inc_slot) {
  const int64_t N = p->N, E = p->E;
  const int nen = p->nen, ndof = p->ndof;
  // node adjacency: union of the nodes of every incident element, sorted
  std::vector<int> adj_ptr(N + 1, 0);
  std::vector<int> adj;
  adj.reserve((size_t)N * 27);
  std::vector<int> mark(N, -1);
  std::vector<int> tmp;
  for (int64_t n = 0; n < N; ++n) {
    tmp.clear();
    for (int k = inc_ptr[n]; k < inc_ptr[n + 1]; ++k) {
      int e = inc_slot[k] / nen;
      for (int b = 0; b < nen; ++b) {
        int m = conn[(size_t)e * nen + b];
        if (mark[m] != (int)n) {
          mark[m] = (int)n;
          tmp.push_back(m);
        }
      }
    }
    std::sort(tmp.begin(), tmp.end());
    if ((int)tmp.size() > p->maxdeg) p->maxdeg = (int)tmp.size();
    adj.insert(adj.end(), tmp.begin(), tmp.end());
    adj_ptr[n + 1] = (int)adj.size();
  }
  const int64_t P = (int64_t)adj.size();
  const int64_t nnz = P * ndof * ndof;
  if (nnz > (int64_t)INT32_MAX) return FOLGB_ERR_INVALID_ARGUMENT;
  // dof-level canonical CSR: row ndof*n+c holds ndof*deg(n) entries,
  // neighbour-major, component-minor (sorted columns).
  const int64_t rows = (int64_t)ndof * N;
  std::vector<int> rowptr(rows + 1, 0);
  std::vector<int> colind(nnz);
  for (int64_t n = 0; n < N; ++n) {
    int deg = adj_ptr[n + 1] - adj_ptr[n];
    for (int c = 0; c < ndof; ++c) {
      int64_t r = ndof * n + c;
      int64_t base = (int64_t)ndof * ndof * adj_ptr[n] + (int64_t)c * ndof * deg;
      rowptr[r] = (int)base;
      for (int j = 0; j < deg; ++j)
        for (int l = 0; l < ndof; ++l) colind[base + (int64_t)j * ndof + l] = ndof * adj[adj_ptr[n] + j] + l;
    }
  }
  rowptr[rows] = (int)nnz;
  std::vector<int> pair_row(P);
  for (int64_t n = 0; n < N; ++n)
    for (int k = adj_ptr[n]; k < adj_ptr[n + 1]; ++k) pair_row[k] = (int)n;
  // element -> pair map, then its stable transpose (pair -> element blocks)
  const int64_t nslots = E * nen * nen;
  std::vector<int> e2p(nslots);
  for (int64_t e = 0; e < E; ++e)
    for (int a = 0; a < nen; ++a) {
      int n = conn[e * nen + a];
      const int* lo = adj.data() + adj_ptr[n];
      const int* hi = adj.data() + adj_ptr[n + 1];
      for (int b = 0; b < nen; ++b) {
        int m = conn[e * nen + b];
        const int* it = std::lower_bound(lo, hi, m);
        e2p[(e * nen + a) * nen + b] = (int)(it - adj.data());
      }
    }
  std::vector<int> pair_ptr(P + 1, 0);
  for (int64_t s = 0; s < nslots; ++s) pair_ptr[e2p[s] + 1]++;
  for (int64_t k = 0; k < P; ++k) pair_ptr[k + 1] += pair_ptr[k];
  std::vector<int> pair_slot(nslots);
  {
    std::vector<int> fill(pair_ptr.begin(), pair_ptr.end() - 1);
    for (int64_t s = 0; s < nslots; ++s) pair_slot[fill[e2p[s]]++] = (int)s;
  }
  int rc;
  if ((rc = upload(&p->d_adj_ptr, adj_ptr.data(), adj_ptr.size()))) return rc;
  if ((rc = upload(&p->d_adj, adj.data(), adj.size()))) return rc;
  if ((rc = upload(&p->d_rowptr, rowptr.data(), rowptr.size()))) return rc;
  if ((rc = upload(&p->d_colind, colind.data(), colind.size()))) return rc;
  if ((rc = upload(&p->d_pair_row, pair_row.data(), pair_row.size()))) return rc;
  if ((rc = upload(&p->d_pair_ptr, pair_ptr.data(), pair_ptr.size()))) return rc;
  if ((rc = upload(&p->d_pair_slot, pair_slot.data(), pair_slot.size()))) return rc;
  p->has_csr = true;
  p->P = P;
  p->nnz = nnz;
  p->rows = rows;
  return FOLGB_OK;
}

int check_physics(const folgb_physics* phys, int& nen, int& dim, int& ndof) {
  if (!phys) return FOLGB_ERR_INVALID_ARGUMENT;
  switch (phys->element_type) {
    case FOLGB_QUAD4: nen = 4; dim = 2; break;
    case FOLGB_HEX8: nen = 8; dim = 3; break;
    case FOLGB_TET4: nen = 4; dim = 3; break;
    default: return FOLGB_ERR_INVALID_ARGUMENT;
  }
  if (phys->physics < FOLGB_THERMAL || phys->physics > FOLGB_NEOHOOKE_SPLIT) return FOLGB_ERR_INVALID_ARGUMENT;
  // the transient element's control is the nodal current temperature field
  if (phys->physics == FOLGB_TRANSIENT_THERMAL &&
      (phys->control_layout != FOLGB_CONTROL_NODAL || !(phys->time_step > 0.0)))
    return FOLGB_ERR_INVALID_ARGUMENT;
  if (phys->control_layout != FOLGB_CONTROL_NODAL && phys->control_layout != FOLGB_CONTROL_ELEMENT)
    return FOLGB_ERR_INVALID_ARGUMENT;
  if (phys->num_gp < 1 || phys->num_gp > 3) return FOLGB_ERR_INVALID_ARGUMENT;
  ndof = (phys->physics == FOLGB_THERMAL || phys->physics == FOLGB_TRANSIENT_THERMAL) ? 1 : dim;
  return FOLGB_OK;
}

}  // namespace folgb

extern "C" int folgb_plan_create(folgb_plan** out, const folgb_physics* phys, const int64_t* conn,
                                 int64_t num_elements, const double* xyz, int64_t num_nodes,
                                 const int64_t* dirichlet_dofs, const double* dirichlet_values,
                                 int64_t num_dirichlet, int32_t build_csr) {
  if (!out) return FOLGB_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int nen, dim, ndof;
  int rc = check_physics(phys, nen, dim, ndof);
  if (rc) return rc;
  if (num_elements <= 0 || num_nodes <= 0 || !conn || !xyz) return FOLGB_ERR_INVALID_ARGUMENT;
  if (num_nodes > (int64_t)INT32_MAX / 4 || num_elements * nen * nen > (int64_t)INT32_MAX)
    return FOLGB_ERR_INVALID_ARGUMENT;
  if (num_dirichlet < 0 || (num_dirichlet > 0 && (!dirichlet_dofs || !dirichlet_values)))
    return FOLGB_ERR_INVALID_ARGUMENT;
  std::vector<int> c32((size_t)num_elements * nen);
  for (int64_t i = 0; i < num_elements * nen; ++i) {
    if (conn[i] < 0 || conn[i] >= num_nodes) return FOLGB_ERR_INVALID_ARGUMENT;
    c32[i] = (int)conn[i];
  }
  const int64_t ndofs = (int64_t)ndof * num_nodes;
  for (int64_t i = 0; i < num_dirichlet; ++i)
    if (dirichlet_dofs[i] < 0 || dirichlet_dofs[i] >= ndofs) return FOLGB_ERR_INVALID_ARGUMENT;

  folgb_plan* p = new folgb_plan();
  p->phys = *phys;
  p->etype = phys->element_type;
  p->physics = phys->physics;
  p->nen = nen;
  p->dim = dim;
  p->ndof = ndof;
  p->E = num_elements;
  p->N = num_nodes;
  p->ctrl_layout = phys->control_layout;
  // kernel_variant >= 2 pins sum-factorised variant (kernel_variant - 2)
  p->hex8_variant = phys->kernel_variant >= 2 ? phys->kernel_variant - 2 : 0;
  if ((rc = fill_material(*phys, dim, p->mat)) || !build_gp_table(p->etype, phys->num_gp, p->h_gp)) {
    delete p;
    return rc ? rc : FOLGB_ERR_INVALID_ARGUMENT;
  }
  std::vector<float4> x4(num_nodes);
  for (int64_t n = 0; n < num_nodes; ++n)
    x4[n] = make_float4((float)xyz[3 * n], (float)xyz[3 * n + 1], (float)xyz[3 * n + 2], 0.f);
  std::vector<int> inc_ptr, inc_slot;
  build_incidence(c32, num_elements, nen, num_nodes, inc_ptr, inc_slot);
  // the device lists hold record indices a*E + e: element results are stored
  // local-node-major, so a warp of consecutive nodes reads consecutive records
  std::vector<int> inc_rec(inc_slot.size());
  for (size_t k = 0; k < inc_slot.size(); ++k)
    inc_rec[k] = (int)((inc_slot[k] % nen) * num_elements + inc_slot[k] / nen);
  // padded copy of the incidence lists for vector loads when every node has
  // at most 4 or 8 incident element slots (structured quad / hex meshes)
  int maxinc = 0;
  for (int64_t n = 0; n < num_nodes; ++n) maxinc = std::max(maxinc, inc_ptr[n + 1] - inc_ptr[n]);
  const int pad = maxinc <= 4 ? 4 : (maxinc <= 8 ? 8 : 0);
  p->inc_pad = pad;
  std::vector<int> inc_padded;
  if (pad) {
    inc_padded.assign((size_t)num_nodes * pad, -1);
    for (int64_t n = 0; n < num_nodes; ++n)
      for (int k = inc_ptr[n]; k < inc_ptr[n + 1]; ++k) inc_padded[(size_t)n * pad + (k - inc_ptr[n])] = inc_rec[k];
  }
  std::vector<unsigned char> dmask(num_nodes, 0);
  std::vector<float> dval(ndofs, 0.f);
  p->dir_dofs.assign(dirichlet_dofs, dirichlet_dofs + num_dirichlet);
  p->dir_vals.assign(dirichlet_values, dirichlet_values + num_dirichlet);
  for (int64_t i = 0; i < num_dirichlet; ++i) {
    int64_t d = dirichlet_dofs[i];
    dmask[d / ndof] |= (unsigned char)(1u << (d % ndof));
    dval[d] = (float)dirichlet_values[i];  // later entries win, as numpy/XLA .at[].set
  }
  // per-element Dirichlet flag: kernels read the nodal masks only for the
  // elements that touch a constrained node (3 % of a 64^3 box)
  std::vector<unsigned char> elem_bc(num_elements, 0);
  for (int64_t e = 0; e < num_elements; ++e)
    for (int a = 0; a < nen; ++a) elem_bc[e] |= dmask[c32[(size_t)e * nen + a]] ? 1 : 0;
  if ((rc = upload(&p->d_conn, c32.data(), c32.size())) || (rc = upload(&p->d_xyz4, x4.data(), x4.size())) ||
      (rc = upload(&p->d_elem_bc, elem_bc.data(), elem_bc.size())) ||
      (rc = upload(&p->d_k0, std::vector<float>(num_nodes, 1.f).data(), (size_t)num_nodes)) ||
      (rc = upload(&p->d_inc_ptr, inc_ptr.data(), inc_ptr.size())) ||
      (rc = upload(&p->d_inc_slot, inc_rec.data(), inc_rec.size())) ||
      (pad && (rc = upload(&p->d_inc_padded, inc_padded.data(), inc_padded.size()))) ||
      (rc = upload(&p->d_dmask, dmask.data(), dmask.size())) || (rc = upload(&p->d_dval, dval.data(), dval.size())) ||
      (rc = upload(&p->d_gp, &p->h_gp, 1))) {
    folgb_plan_destroy(p);
    return rc;
  }
  if (build_csr && (rc = build_csr_tables(p, c32, inc_ptr, inc_slot))) {
    folgb_plan_destroy(p);
    return rc;
  }
  // tile tables of the tile-local fused kernel (hex8 elasticity, 2x2x2 Gauss)
  if (p->etype == FOLGB_HEX8 && p->physics == FOLGB_ELASTIC && phys->num_gp == 2 &&
      (rc = build_tile_tables(p, c32, xyz, dmask, elem_bc))) {
    folgb_plan_destroy(p);
    return rc;
  }
  // patches of 6 tetrahedra on 8 nodes (the 6-tet split of a hexahedron)
  if ((rc = build_tet_patches(p, c32))) {
    folgb_plan_destroy(p);
    return rc;
  }
  // box kernels when every element is the same axis-aligned box
  if ((rc = build_uniform_box(p, x4, c32, dmask))) {
    folgb_plan_destroy(p);
    return rc;
  }
  noalloc_prepare_current_device();
  *out = p;
  return FOLGB_OK;
}

extern "C" int folgb_plan_destroy(folgb_plan* p) {
  if (!p) return FOLGB_OK;
  void* ptrs[] = {p->d_conn, p->d_xyz4, p->d_inc_ptr, p->d_inc_slot, p->d_inc_padded, p->d_dmask, p->d_elem_bc,
                  p->d_k0, p->d_dval, p->d_gp,
                  p->d_adj_ptr, p->d_adj, p->d_rowptr, p->d_colind, p->d_pair_row, p->d_pair_ptr,
                  p->d_pair_slot, p->d_box_layer_bc};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  free_tile_tables(p);
  free_tet_patches(p);
  free_krylov_graphs(p);
  delete p;
  return FOLGB_OK;
}

extern "C" int folgb_plan_info(const folgb_plan* p, int64_t* ndof_per_node, int64_t* total_dofs,
                               int64_t* csr_rows, int64_t* csr_nnz) {
  if (!p) return FOLGB_ERR_INVALID_ARGUMENT;
  if (ndof_per_node) *ndof_per_node = p->ndof;
  if (total_dofs) *total_dofs = (int64_t)p->ndof * p->N;
  if (csr_rows) *csr_rows = p->has_csr ? p->rows : 0;
  if (csr_nnz) *csr_nnz = p->has_csr ? p->nnz : 0;
  return FOLGB_OK;
}

extern "C" int folgb_plan_features(const folgb_plan* p, int32_t* features) {
  if (!p || !features) return FOLGB_ERR_INVALID_ARGUMENT;
  *features = (p->tiles > 0 ? FOLGB_FEATURE_TILES : 0) | (p->box_valid ? FOLGB_FEATURE_UNIFORM_BOX : 0) |
              (p->box_grid ? FOLGB_FEATURE_BOX_GRID : 0) | (p->n_patches > 0 ? FOLGB_FEATURE_TET_PATCHES : 0);
  return FOLGB_OK;
}

extern "C" int folgb_plan_set_dirichlet_values(folgb_plan* p, const double* values, double load_increment) {
  if (!p || (!values && !p->dir_dofs.empty())) return FOLGB_ERR_INVALID_ARGUMENT;
  for (size_t i = 0; i < p->dir_dofs.size(); ++i) p->dir_vals[i] = values[i];
  // rebuild the dense value table (later entries win)
  std::vector<float> dval((size_t)p->ndof * p->N, 0.f);
  for (size_t i = 0; i < p->dir_dofs.size(); ++i) dval[p->dir_dofs[i]] = (float)(load_increment * values[i]);
  FOLGB_CUDA_TRY(cudaMemcpy(p->d_dval, dval.data(), dval.size() * sizeof(float), cudaMemcpyHostToDevice));
  return FOLGB_OK;
}

extern "C" int folgb_plan_set_nodal_field(folgb_plan* p, const double* values) {
  if (!p || !values) return FOLGB_ERR_INVALID_ARGUMENT;
  std::vector<float> v(p->N);
  for (int64_t n = 0; n < p->N; ++n) v[n] = (float)values[n];
  FOLGB_CUDA_TRY(cudaMemcpy(p->d_k0, v.data(), v.size() * sizeof(float), cudaMemcpyHostToDevice));
  return FOLGB_OK;
}

extern "C" int folgb_csr_pattern(const folgb_plan* p, int32_t* indptr, int32_t* indices, void* stream) {
  if (!p || !indptr || !indices) return FOLGB_ERR_INVALID_ARGUMENT;
  if (!p->has_csr) return FOLGB_ERR_NO_PATTERN;
  cudaStream_t s = (cudaStream_t)stream;
  FOLGB_CUDA_TRY(cudaMemcpyAsync(indptr, p->d_rowptr, (p->rows + 1) * sizeof(int), cudaMemcpyDeviceToDevice, s));
  FOLGB_CUDA_TRY(cudaMemcpyAsync(indices, p->d_colind, p->nnz * sizeof(int), cudaMemcpyDeviceToDevice, s));
  return FOLGB_OK;
}
