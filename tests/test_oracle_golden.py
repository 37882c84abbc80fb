"""The FP64 oracle against the reference's own golden vectors (CPU only)."""
import numpy as np
import pytest

from conftest import arr, golden
from oracle import fe_oracle as fo

NGP = {"tet4": 1, "hex8": 2, "quad4": 2}


@pytest.mark.parametrize("etype", ["tet4", "hex8", "quad4"])
def test_linear_elastic_element_golden(etype):
    """tests/unit/test_mechanical_loss.py: K_e, r_e (E=1, nu=0.3, controls 1, u 1)."""
    g = golden("mechanical_linear.json")[etype]
    nen, dim = fo.ELEMENTS[etype]
    en, re, K, dE = fo.linear_elastic_element(etype, arr(g["xyz"]), np.ones(nen), np.ones(nen * dim), NGP[etype],
                                              1.0, 0.3, arr(g["body_force"]).ravel())
    np.testing.assert_allclose(K, arr(g["stiffness"]), rtol=1e-5, atol=1e-6)
    # the reference itself checks the tet residual at rtol 1e-4 (test_mechanical_loss.py:38-39)
    np.testing.assert_allclose(re, arr(g["residual"]), rtol=1e-4 if etype == "tet4" else 1e-5, atol=1e-6)


@pytest.mark.parametrize("etype", ["tet4", "hex8"])
def test_saint_venant_at_zero_strain_is_the_linear_golden(etype):
    """test_saint_venant_mechanical_loss.py evaluates the Saint-Venant element
    at u = 1 (a rigid translation: F = I, E = 0).  There its tangent is the
    linear-elastic stiffness (3-D Lame constants) and its residual -F_e, so
    the linear-elastic golden vectors (test_mechanical_loss.py, same E, nu and
    body force) pin it."""
    g = golden("mechanical_linear.json")[etype]
    nen, dim = fo.ELEMENTS[etype]
    en, re, K, fint, dE = fo.saint_venant_element(etype, arr(g["xyz"]), np.ones(nen), np.ones(nen * dim), NGP[etype],
                                                  0.3, arr(g["body_force"]).ravel())
    np.testing.assert_allclose(K, arr(g["stiffness"]), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(re, arr(g["residual"]), rtol=1e-4 if etype == "tet4" else 1e-5, atol=1e-6)
    assert abs(en) < 1e-12 and np.abs(fint).max() < 1e-12


@pytest.mark.parametrize("etype", ["tet4", "hex8", "quad4"])
def test_neohooke_element_golden(etype):
    """tests/unit/test_neo_hooke_mechanical_loss_AD.py: K_e = jacfwd(r_e), r_e."""
    g = golden("neohooke_ad.json")[etype]
    nen, dim = fo.ELEMENTS[etype]
    en, re, K, fc, dE = fo.neohooke_element(etype, arr(g["xyz"]), np.ones(nen), np.ones(nen * dim), NGP[etype], 0.3,
                                            arr(g["body_force"]).ravel(), "reference")
    np.testing.assert_allclose(K, arr(g["stiffness"]), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(re, arr(g["residual"]), rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("etype", ["tet4", "hex8", "quad4"])
def test_neohooke_split_element_golden(etype):
    """tests/unit/test_neo_hooke_mechanical_loss.py (the non-AD element of
    mechanical_neohooke.py): K_e = B^T C B + geometric stiffness, r_e, at u = 1."""
    g = golden("neohooke.json")[etype]
    nen, dim = fo.ELEMENTS[etype]
    en, re, K, fint, dE = fo.neohooke_split_element(etype, arr(g["xyz"]), np.ones(nen), np.ones(nen * dim),
                                                    NGP[etype], g["poisson_ratio"], arr(g["body_force"]).ravel())
    np.testing.assert_allclose(K, arr(g["stiffness"]), rtol=g["rtol"], atol=g["atol"])
    np.testing.assert_allclose(re, arr(g["residual"]).ravel(), rtol=g["rtol"], atol=g["atol"])
    # u = 1 is a rigid translation: stress-free, so r_e = -F_e
    assert abs(en) < 1e-12 and np.abs(fint).max() < 1e-12


@pytest.mark.parametrize("etype", ["quad4", "tet4", "hex8"])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_geometry_golden(etype, order):
    """tests/unit/test_geometries.py: Gauss rules, N, dN/dxi, J, dN/dx."""
    G = golden("geometries.json")[etype]
    g = G[f"gi{order}"]
    pts, w = fo.gauss_rule(etype, order)
    ep = arr(g["points"])
    np.testing.assert_allclose(pts[:, : ep.shape[1]], ep, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(w, arr(g["weights"]), rtol=1e-5, atol=1e-6)
    if "N" in g:
        X = arr(G["xyz"])
        N = np.array([fo.shape_values(etype, p) for p in pts])
        np.testing.assert_allclose(N, arr(g["N"]).reshape(N.shape), rtol=1e-5, atol=1e-6)
        dN = np.array([fo.shape_local_grads(etype, p) for p in pts])
        np.testing.assert_allclose(dN, arr(g["dN_dxi"]).reshape(dN.shape), rtol=1e-5, atol=1e-6)
        J = np.array([fo.jacobian(etype, X, p) for p in pts])
        np.testing.assert_allclose(J, arr(g["jacobian"]).reshape(J.shape), rtol=1e-5, atol=1e-6)
        dx = np.array([fo.global_grads(etype, X, p)[0] for p in pts])
        np.testing.assert_allclose(dx, arr(g["dN_dx"]).reshape(dx.shape), rtol=1e-5, atol=1e-6)


def test_gauss_order_4_not_implemented():
    """test_geometries.py:366-371: orders 4 and 5 raise NotImplementedError."""
    for order in (4, 5):
        with pytest.raises(NotImplementedError):
            fo.gauss_rule("quad4", order)


def test_sensitivity_golden():
    """tests/unit/test_sensitivity_analysis.py: transposed BC Jacobian row,
    adjoint RHS, nodal control and shape derivatives on a 3x3-node quad mesh."""
    S = golden("sensitivity_quad4.json")
    xyz, conn, sets = fo.square_mesh(S["mesh_L"], S["mesh_N"])
    L = fo.FELossOracle("quad4", "elastic", xyz, conn, dirichlet=S["bc"], node_sets=sets, num_gp=2,
                        young=S["young_modulus"], nu=S["poisson_ratio"])
    R = fo.QuadResponseOracle(L)
    u, K, adj = arr(S["u"]), arr(S["control"]), arr(S["adjoint_u"])
    A, rhs = R.adjoint_jacobian_and_rhs(K, u)
    tol = dict(rtol=S["rtol"], atol=S["atol"])
    np.testing.assert_allclose(A.toarray()[8], arr(S["jacobian_row8"]), **tol)
    np.testing.assert_allclose(rhs, arr(S["rhs"]), **tol)
    np.testing.assert_allclose(R.nodal_control_derivatives(K, u, adj), arr(S["control_derivatives"]), **tol)
    np.testing.assert_allclose(R.nodal_shape_derivatives(K, u, adj), arr(S["shape_derivatives"]), **tol)


@pytest.mark.parametrize("etype", ["tet4", "hex8"])
def test_transient_thermal_element_golden(etype):
    """tests/unit/test_nonlinear_transient_thermal.py: ComputeElement with
    T_current = 1, T_next = 0, k0 = 1 (rho = cp = 1, beta = 1.5, dt = 0.005)."""
    G = golden("transient_thermal.json")
    g = G[etype]
    nen = fo.ELEMENTS[etype][0]
    en, re, K, dEn, dEc = fo.transient_thermal_element(etype, arr(g["xyz"]), np.ones(nen), np.zeros(nen), np.ones(nen),
                                                       NGP[etype], G["rho"] * G["cp"], G["time_step"], G["beta"],
                                                       G["c"])
    np.testing.assert_allclose(K, arr(g["stiffness"]), rtol=G["rtol"], atol=G["atol"])
    np.testing.assert_allclose(re, arr(g["residual"]), rtol=G["rtol"], atol=G["atol"])
