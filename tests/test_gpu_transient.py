"""Implicit-Euler transient heat conduction (transient_thermal.py) through the
CUDA path: the reference's element golden vectors, loss + adjoint (the
gradients with respect to the next AND the current temperature field), CSR
tangent and residual, and Newton time steps against the FP64 oracle.
Tolerance 1e-5 relative (Frobenius)."""
import numpy as np
import pytest

from conftest import arr, golden
from gpu_cases import make_mesh, rel_fro
from oracle import fe_oracle as fo

pytestmark = pytest.mark.gpu
TOL = 1e-5
NAMES = {"quad4": "quad", "hex8": "hexahedron", "tet4": "tetra"}


def _pair(etype, n, beta=1.5, c=1.0, dt=0.01, seed=91):
    from folax_gb300 import loss as L
    m = make_mesh(etype, n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    k0 = 0.5 + rng.random(m.GetNumberOfNodes())
    bc = {"T": {"left": 1.0, "right": 0.0}} if etype == "quad4" else {"T": {"bottom": 1.0, "top": 0.0}}
    settings = {"dirichlet_bc_dict": bc, "material_dict": {"rho": 1.2, "cp": 0.9, "beta": beta, "k0": k0},
                "time_integration_dict": {"method": "implicit-euler", "time_step": dt}, "c": c}
    cls = {"quad4": L.TransientThermalLoss2DQuad, "hex8": L.TransientThermalLoss3DHexa,
           "tet4": L.TransientThermalLoss3DTetra}[etype]
    gl = cls("tt", dict(settings), m)
    gl.Initialize()
    ol = fo.FELossOracle(etype, "transient_thermal", m.nodes_coordinates, m.elements_nodes[NAMES[etype]],
                         dirichlet=bc, node_sets=m.node_sets, c=c, rho_cp=1.2 * 0.9, time_step=dt,
                         material_beta=beta, k0=k0)
    return m, gl, ol


@pytest.mark.parametrize("etype", ["tet4", "hex8"])
def test_element_golden_on_gpu(cuda, etype):
    from folax_gb300 import loss as L
    G = golden("transient_thermal.json")
    g = G[etype]
    nen = fo.ELEMENTS[etype][0]
    mesh = make_mesh(etype, 1)
    cls = L.TransientThermalLoss3DTetra if etype == "tet4" else L.TransientThermalLoss3DHexa
    loss = cls("tt", {"dirichlet_bc_dict": {"T": {}},
                      "material_dict": {"rho": G["rho"], "cp": G["cp"], "beta": G["beta"], "c": G["c"]},
                      "time_integration_dict": {"method": "implicit-euler", "time_step": G["time_step"]}}, mesh)
    loss.Initialize()
    en, re, K = loss.ComputeElement(arr(g["xyz"]), np.ones(nen), np.zeros(nen), np.ones(nen))
    np.testing.assert_allclose(K, arr(g["stiffness"]), rtol=G["rtol"], atol=1e-9)
    np.testing.assert_allclose(re, arr(g["residual"]), rtol=G["rtol"], atol=1e-9)


@pytest.mark.parametrize("etype,n", [("quad4", 8), ("hex8", 3), ("tet4", 3)])
@pytest.mark.parametrize("beta,c", [(0.0, 1.0), (1.5, 1.0), (0.8, 2.0)])
def test_loss_adjoint_matches_oracle(cuda, etype, n, beta, c):
    m, gl, ol = _pair(etype, n, beta, c)
    rng = np.random.default_rng(92)
    Tc = 0.3 + 0.5 * rng.random((2, m.GetNumberOfNodes()))
    Tn = 0.3 + 0.5 * rng.random((2, m.GetNumberOfNodes()))
    a = gl.ComputeBatchLossAndGrad(Tc, Tn)
    o = ol.batch_loss_and_grads(Tc, Tn)
    gl.CheckDeviceStatus()
    for x, z in zip(a[2:], o[2:]):
        assert rel_fro(x.cpu().numpy(), z) < TOL


@pytest.mark.parametrize("etype,n", [("quad4", 6), ("hex8", 3), ("tet4", 3)])
@pytest.mark.parametrize("transpose", [False, True])
def test_tangent_and_residual_match_oracle(cuda, etype, n, transpose):
    m, gl, ol = _pair(etype, n, 1.5, 2.0)
    rng = np.random.default_rng(93)
    Tc = 0.3 + 0.5 * rng.random(m.GetNumberOfNodes())
    Tn = ol.full_dof_vector(0.3 + 0.5 * rng.random(m.GetNumberOfNodes()))
    jac, R = gl.ComputeJacobianMatrixAndResidualVector(Tc, Tn, transpose_jacobian=transpose)
    A, Ro = ol.csr(Tc, Tn, transpose=transpose)
    assert rel_fro(jac.data.cpu().numpy(), A.data) < TOL
    assert rel_fro(R.cpu().numpy(), Ro) < TOL


def test_newton_time_steps_match_oracle(cuda):
    """Three implicit-Euler steps of the nonlinear problem, each a Newton solve
    with T_current the previous step's result."""
    from folax_gb300.solvers import FiniteElementNonLinearResidualBasedSolver
    m, gl, ol = _pair("quad4", 10, 1.5, 1.0, dt=0.02)
    solver = FiniteElementNonLinearResidualBasedSolver("nl", gl, {
        "linear_solver_settings": {"solver": "JAX-bicgstab", "tol": 1e-10, "maxiter": 5000, "vector_precision": "fp64"},
        "nonlinear_solver_settings": {"load_incr": 1, "maxiter": 10, "abs_tol": 1e-9, "rel_tol": 1e-9}})
    solver.Initialize()
    T = np.zeros(m.GetNumberOfNodes())
    To = T.copy()
    for _ in range(3):
        T = solver.Solve(T, T).double().cpu().numpy()
        To, _ = fo.newton_solve(ol, To, To, load_incr=1, maxiter=10, abs_tol=1e-9, rel_tol=1e-9)
    assert rel_fro(T, To) < TOL
