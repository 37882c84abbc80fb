"""Oracle self-consistency (CPU): gradient definitions by central finite
differences and complex step, CSR canonical form, PCG vs direct solve."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import fe_oracle as fo
from folax_gb300 import mesh as M, fields


def _small(etype, physics, n=3, seed=0, layout="nodal", exponent=1.0, bf=None):
    rng = np.random.default_rng(seed)
    if etype == "quad4":
        m = M.create_2D_square_mesh(1.0, n + 1)
        conn = m.elements_nodes["quad"]
        dirichlet = {"T": {"left": 1.0, "right": 0.0}} if physics == "thermal" else \
            {"Ux": {"left": 0.0, "right": 0.05}, "Uy": {"left": 0.0}}
    else:
        m = M.create_3D_box_mesh(n, n, n)
        if etype == "tet4":
            m = M.split_hex_to_tets(m)
        conn = m.elements_nodes["hexahedron" if etype == "hex8" else "tetra"]
        dirichlet = {"T": {"bottom": 1.0, "top": 0.0}} if physics == "thermal" else \
            {"Ux": {"bottom": 0.0}, "Uy": {"bottom": 0.0}, "Uz": {"bottom": 0.0, "top": 0.05}}
    xyz = m.nodes_coordinates + 0.02 * rng.standard_normal(m.nodes_coordinates.shape) * (1 if etype != "quad4" else np.array([1, 1, 0]))
    L = fo.FELossOracle(etype, physics, xyz, conn, dirichlet=dirichlet, node_sets=m.node_sets,
                        exponent=exponent, control_layout=layout, body_force=bf)
    nctrl = len(conn) if layout == "element" else len(xyz)
    ctrl = 0.5 + rng.random(nctrl)
    u = 0.05 * rng.standard_normal(L.total_dofs)
    return L, ctrl, u


@pytest.mark.parametrize("etype,physics", [("quad4", "thermal"), ("hex8", "elastic"), ("tet4", "neohooke"),
                                           ("quad4", "elastic"), ("hex8", "neohooke"), ("tet4", "thermal")])
@pytest.mark.parametrize("layout", ["nodal", "element"])
def test_loss_gradients_fd(etype, physics, layout):
    """dLoss/du (free dofs) and dLoss/dcontrol against FP64 central differences
    of the loss value; for thermal/elastic the u-gradient is the stop_gradient
    residual, checked as the FD of 0.5 u^T K u (+ linear part) instead."""
    L, ctrl, u = _small(etype, physics, layout=layout, exponent=1.3 if physics != "neohooke" else 1.0)
    mean, _, losses, du, dc = L.batch_loss_and_grads(ctrl[None], u[None])
    h = 1e-6
    rng = np.random.default_rng(1)
    # control gradient: FD of the loss value
    for _ in range(3):
        d = rng.standard_normal(ctrl.shape)
        fp = L.batch_loss_and_grads((ctrl + h * d)[None], u[None])[0]
        fm = L.batch_loss_and_grads((ctrl - h * d)[None], u[None])[0]
        np.testing.assert_allclose((fp - fm) / (2 * h), dc[0] @ d, rtol=2e-6, atol=1e-12)
    if physics == "neohooke":
        for _ in range(3):
            d = rng.standard_normal(u.shape)
            d[L.dirichlet_indices] = 0
            fp = L.batch_loss_and_grads(ctrl[None], (u + h * d)[None])[0]
            fm = L.batch_loss_and_grads(ctrl[None], (u - h * d)[None])[0]
            np.testing.assert_allclose((fp - fm) / (2 * h), du[0] @ d, rtol=2e-6, atol=1e-12)
    assert np.all(du[0][L.dirichlet_indices] == 0)


def test_neohooke_reference_shear_is_not_energy_gradient():
    """The reference residual doubles the shear stresses (utils.py:45-56); the
    consistent one is the energy gradient."""
    L, ctrl, u = _small("hex8", "neohooke", n=1)
    X, de, ue, _ = L._gather(ctrl, L.full_dof_vector(u))
    en, re_ref, _, fc, _ = fo.neohooke_element("hex8", X, de, ue, 2, 0.3, None, "reference", want_tangent=False)
    _, re_con, _, _, _ = fo.neohooke_element("hex8", X, de, ue, 2, 0.3, None, "consistent", want_tangent=False)
    np.testing.assert_allclose(re_con, fc, rtol=1e-12, atol=1e-14)
    assert np.abs(re_ref - re_con).max() > 1e-3 * np.abs(re_con).max()


@pytest.mark.parametrize("mode", ["reference", "consistent"])
def test_neohooke_tangent_complex_step(mode):
    L, ctrl, u = _small("tet4", "neohooke", n=1)
    X, de, ue, _ = L._gather(ctrl, L.full_dof_vector(u))
    _, _, K, _, _ = fo.neohooke_element("tet4", X[:2], de[:2], ue[:2], 1, 0.3, None, mode)
    for e in range(2):
        Kc = fo._complex_step(lambda v: fo.neohooke_element("tet4", X[e], de[e], v, 1, 0.3, None, mode,
                                                            want_tangent=False)[1], ue[e])
        np.testing.assert_allclose(K[e], Kc, rtol=1e-9, atol=1e-12)


def test_csr_canonical_and_bc_rows():
    L, ctrl, u = _small("hex8", "elastic", n=2)
    A, R = L.csr(ctrl, L.full_dof_vector(u))
    assert A.has_canonical_format
    d = A.toarray()
    for i in L.dirichlet_indices:
        row = d[i].copy()
        assert row[i] != 0
        row[i] = 0
        assert np.all(row == 0)
    assert np.all(R[L.dirichlet_indices] == 0)


def test_pcg_matches_direct():
    L, ctrl, u = _small("hex8", "elastic", n=3)
    uf = L.full_dof_vector(np.zeros(L.total_dofs))
    A, R = L.csr(ctrl, uf)
    x_d = fo.direct_solve(A, -R)
    x_p, it, rel = fo.jacobi_pcg(A, -R, rtol=1e-12)
    assert rel <= 1e-12
    np.testing.assert_allclose(x_p, x_d, rtol=1e-8, atol=1e-12 * np.abs(x_d).max())


def test_newton_neohooke_converges():
    L, ctrl, u = _small("tet4", "neohooke", n=2)
    u1, hist = fo.newton_solve(L, ctrl, np.zeros(L.total_dofs), load_incr=2, maxiter=10)
    assert hist[-1][2] < 1e-8 or hist[-1][3] < 1e-8


@pytest.mark.parametrize("etype", ["tet4", "hex8", "quad4"])
@pytest.mark.parametrize("element", ["saint_venant_element", "neohooke_split_element"])
def test_hyperelastic_element_consistency(etype, element):
    """Saint-Venant and split neo-Hooke elements: internal force = d energy / d u
    and tangent = d residual / d u (complex step), energy control derivative =
    d energy / d e."""
    elem = getattr(fo, element)
    rng = np.random.default_rng(9)
    nen, dim = fo.ELEMENTS[etype]
    if etype == "quad4":
        X = np.array([[0.0, 0.0, 0.0], [1.1, 0.1, 0.0], [1.0, 0.9, 0.0], [0.1, 1.2, 0.0]])
    elif etype == "tet4":
        X = np.array([[0.0, 0.0, 0.0], [1.0, 0.1, 0.0], [0.1, 1.0, 0.1], [0.0, 0.2, 1.1]])
    else:
        X = np.array(fo._HEX_SIGNS) * 0.5 + 0.5 + 0.05 * rng.standard_normal((8, 3))
    de = 0.5 + rng.random(nen)
    ue = 0.1 * rng.standard_normal(nen * dim)
    bf = np.array([0.3, -0.2, 0.1])
    en, re, K, fint, dEn = elem(etype, X, de, ue, None, 0.3, bf)
    dE_du = fo._complex_step(lambda v: elem(etype, X, de, v, None, 0.3, bf, False)[0], ue)
    np.testing.assert_allclose(fint, dE_du, rtol=1e-10, atol=1e-12)
    dR = fo._complex_step(lambda v: elem(etype, X, de, v, None, 0.3, bf, False)[1], ue)
    np.testing.assert_allclose(K, dR, rtol=1e-10, atol=1e-12)
    dE_de = fo._complex_step(lambda d: elem(etype, X, d, ue, None, 0.3, bf, False)[0], de)
    np.testing.assert_allclose(dEn, dE_de, rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("etype", ["tet4", "hex8", "quad4"])
@pytest.mark.parametrize("beta,c", [(0.0, 1.0), (1.5, 1.0), (0.7, 2.0)])
def test_transient_thermal_consistency(etype, beta, c):
    """Transient thermal element: dEnergy/dTn and dEnergy/dTc are the
    derivatives of the energy value, and the tangent is (d residual / d Tn)^T."""
    rng = np.random.default_rng(11)
    nen, dim = fo.ELEMENTS[etype]
    X = {"quad4": np.array([[0.0, 0.0, 0.0], [1.1, 0.1, 0.0], [1.0, 0.9, 0.0], [0.1, 1.2, 0.0]]),
         "tet4": np.array([[0.0, 0.0, 0.0], [1.0, 0.1, 0.0], [0.1, 1.0, 0.1], [0.0, 0.2, 1.1]]),
         "hex8": np.array(fo._HEX_SIGNS) * 0.5 + 0.5 + 0.05 * rng.standard_normal((8, 3))}[etype]
    Tc, Tn, k0 = rng.random(nen), 0.5 + rng.random(nen), 0.5 + rng.random(nen)
    args = (None, 2 if etype != "tet4" else 1, 1.3, 0.01, beta, c)

    def f(tc, tn):
        return fo.transient_thermal_element(etype, X, tc, tn, k0, *args[1:])
    en, re, K, dEn, dEc = f(Tc, Tn)
    np.testing.assert_allclose(dEn, fo._complex_step(lambda v: f(Tc, v)[0], Tn), rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(dEc, fo._complex_step(lambda v: f(v, Tn)[0], Tc), rtol=1e-10, atol=1e-12)
    # the reference's tangent writes the conductivity-derivative term as
    # N_a (grad T . grad N_b) (transient_thermal.py:64), the transpose of
    # d r_a / d T_b; Me and the conductivity term are symmetric, so the whole
    # matrix is the transpose of the exact Jacobian (equal when beta = 0)
    np.testing.assert_allclose(K, fo._complex_step(lambda v: f(Tc, v)[1], Tn).T, rtol=1e-10, atol=1e-12)
