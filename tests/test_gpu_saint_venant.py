"""Saint-Venant-Kirchhoff elements (mechanical_saint_venant.py) through the
CUDA path: the element at zero strain against the reference's linear-elastic
golden vectors, loss + adjoint, CSR tangent and residual, and Newton against
the FP64 oracle.  Tolerance 1e-5 relative (Frobenius)."""
import numpy as np
import pytest

from conftest import arr, golden
from gpu_cases import bc_dict, gpu_loss, make_mesh, oracle_loss, rel_fro
from oracle import fe_oracle as fo

pytestmark = pytest.mark.gpu
TOL = 1e-5
NGP = {"tet4": 1, "hex8": 2, "quad4": 2}


def _settings(etype, layout="nodal", bf=None):
    s = {"dirichlet_bc_dict": bc_dict(etype, "saint_venant"),
         "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3}, "control_layout": layout}
    if bf is not None:
        s["body_foce"] = bf
    return s


@pytest.mark.parametrize("etype", ["tet4", "hex8"])
def test_zero_strain_element_is_the_linear_golden(cuda, etype):
    from folax_gb300 import loss as L
    g = golden("mechanical_linear.json")[etype]
    nen, dim = fo.ELEMENTS[etype]
    mesh = make_mesh(etype, 1)
    cls = L.SaintVenantMechanicalLoss3DTetra if etype == "tet4" else L.SaintVenantMechanicalLoss3DHexa
    loss = cls("svk", {"dirichlet_bc_dict": {}, "material_dict": {"young_modulus": 1, "poisson_ratio": 0.3},
                       "body_foce": arr(g["body_force"]).ravel().tolist()}, mesh)
    loss.Initialize()
    en, re, K = loss.ComputeElement(arr(g["xyz"]), np.ones(nen), np.ones(nen * dim))
    np.testing.assert_allclose(K, arr(g["stiffness"]), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(re, arr(g["residual"]), rtol=1e-4 if etype == "tet4" else 1e-5, atol=1e-6)


@pytest.mark.parametrize("etype,n", [("tet4", 3), ("hex8", 3), ("quad4", 6)])
@pytest.mark.parametrize("layout", ["nodal", "element"])
def test_loss_adjoint_matches_oracle(cuda, etype, n, layout):
    m = make_mesh(etype, n, seed=81)
    s = _settings(etype, layout, [0.1, -0.2, 0.3])
    gl, ol = gpu_loss(etype, "saint_venant", m, s), oracle_loss(etype, "saint_venant", m, s)
    rng = np.random.default_rng(82)
    ctrl = 0.5 + rng.random((2, gl.GetNumberOfControls()))
    u = (0.2 / n) * rng.standard_normal((2, gl.GetTotalNumberOfDOFs()))
    a = gl.ComputeBatchLossAndGrad(ctrl, u)
    o = ol.batch_loss_and_grads(ctrl, u)
    gl.CheckDeviceStatus()
    for x, z in zip(a[2:], o[2:]):
        assert rel_fro(x.cpu().numpy(), z) < TOL


@pytest.mark.parametrize("etype,n", [("tet4", 3), ("hex8", 3), ("quad4", 5)])
@pytest.mark.parametrize("transpose", [False, True])
def test_tangent_and_residual_match_oracle(cuda, etype, n, transpose):
    m = make_mesh(etype, n, seed=83)
    s = _settings(etype, "nodal", [0.05, 0.1, -0.1])
    gl, ol = gpu_loss(etype, "saint_venant", m, s), oracle_loss(etype, "saint_venant", m, s)
    rng = np.random.default_rng(84)
    ctrl = 0.5 + rng.random(gl.GetNumberOfControls())
    u = ol.full_dof_vector((0.2 / n) * rng.standard_normal(gl.GetTotalNumberOfDOFs()))
    jac, R = gl.ComputeJacobianMatrixAndResidualVector(ctrl, u, transpose_jacobian=transpose)
    A, Ro = ol.csr(ctrl, u, transpose=transpose)
    assert np.array_equal(jac.indptr.cpu().numpy(), A.indptr) and np.array_equal(jac.indices.cpu().numpy(), A.indices)
    assert rel_fro(jac.data.cpu().numpy(), A.data) < TOL
    assert rel_fro(R.cpu().numpy(), Ro) < TOL


@pytest.mark.parametrize("etype,n", [("hex8", 3), ("quad4", 6)])
def test_newton_matches_oracle(cuda, etype, n):
    from folax_gb300.solvers import FiniteElementNonLinearResidualBasedSolver
    m = make_mesh(etype, n, seed=85)
    s = _settings(etype, "nodal")
    gl, ol = gpu_loss(etype, "saint_venant", m, s), oracle_loss(etype, "saint_venant", m, s)
    ctrl = 0.5 + np.random.default_rng(86).random(gl.GetNumberOfControls())
    solver = FiniteElementNonLinearResidualBasedSolver("nl", gl, {
        "linear_solver_settings": {"solver": "JAX-bicgstab", "tol": 1e-10, "maxiter": 5000, "vector_precision": "fp64"},
        "nonlinear_solver_settings": {"load_incr": 2, "maxiter": 10, "abs_tol": 1e-7, "rel_tol": 1e-8}})
    solver.Initialize()
    x = solver.Solve(ctrl, np.zeros(ol.total_dofs)).double().cpu().numpy()
    xo, _ = fo.newton_solve(ol, ctrl, np.zeros(ol.total_dofs), load_incr=2, maxiter=10, abs_tol=1e-7, rel_tol=1e-8)
    assert rel_fro(x, xo) < TOL
