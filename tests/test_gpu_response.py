"""Adjoint sensitivities on the GPU (FiniteElementResponse, fe_response.py and
AdjointFiniteElementSolver, adjoint_fe_solver.py): the reference's golden
vectors (tests/unit/test_sensitivity_analysis.py) through the CUDA path, and
polynomial responses on every element type against the complex-step oracle.
Tolerances: the golden test's own (rtol = atol = 1e-5); 1e-5 relative
(Frobenius) against the oracle."""
import numpy as np
import pytest

from conftest import arr, golden
from gpu_cases import bc_dict, gpu_loss, make_mesh, oracle_loss, rel_fro
from oracle import fe_oracle as fo

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _response(loss, formula, control_name, nctrl):
    from folax_gb300.fields import IdentityControl
    from folax_gb300.response import FiniteElementResponse
    r = FiniteElementResponse("resp", formula, loss, IdentityControl(control_name, {}, nctrl))
    r.Initialize()
    return r


def test_sensitivity_golden_on_gpu(cuda):
    from folax_gb300.loss import MechanicalLoss2DQuad
    from folax_gb300.mesh import create_2D_square_mesh
    S = golden("sensitivity_quad4.json")
    mesh = create_2D_square_mesh(S["mesh_L"], S["mesh_N"])
    loss = MechanicalLoss2DQuad("m", {"dirichlet_bc_dict": S["bc"], "num_gp": S["num_gp"],
                                      "material_dict": {"young_modulus": S["young_modulus"],
                                                        "poisson_ratio": S["poisson_ratio"]}}, mesh)
    loss.Initialize()
    resp = _response(loss, S["response_formula"], "E", mesh.GetNumberOfNodes())
    u, K, adj = arr(S["u"]), arr(S["control"]), arr(S["adjoint_u"])
    tol = dict(rtol=S["rtol"], atol=S["atol"])
    jac, rhs = resp.ComputeAdjointJacobianMatrixAndRHSVector(K, u)
    np.testing.assert_allclose(jac.todense()[8], arr(S["jacobian_row8"]), **tol)
    np.testing.assert_allclose(rhs.cpu().numpy(), arr(S["rhs"]), **tol)
    np.testing.assert_allclose(resp.ComputeAdjointNodalControlDerivatives(K, u, adj).cpu().numpy(),
                               arr(S["control_derivatives"]), **tol)
    np.testing.assert_allclose(resp.ComputeAdjointNodalShapeDerivatives(K, u, adj).cpu().numpy(),
                               arr(S["shape_derivatives"]), **tol)


CASES = [("hex8", "elastic", 3, "nodal", "E*U[0]**2 + 0.5*U[2] - E**2*U[1]*U[2]"),
         ("tet4", "elastic", 3, "element", "(E - 0.3)*U[2]**2"),
         ("quad4", "elastic", 5, "nodal", "E**3*U[1] + U[0]*U[1]"),
         ("quad4", "thermal", 6, "nodal", "K*T[0]**2 - 0.25*K**2"),
         ("hex8", "thermal", 3, "element", "K**2*T[0]"),
         ("tet4", "thermal", 2, "nodal", "T[0]**3 + K*T[0]")]


@pytest.mark.parametrize("etype,physics,n,layout,formula", CASES)
def test_response_and_sensitivities_match_oracle(cuda, etype, physics, n, layout, formula):
    from folax_gb300.response import parse_response_formula
    m = make_mesh(etype, n, seed=71)
    s = {"dirichlet_bc_dict": bc_dict(etype, physics), "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3},
         "control_layout": layout}
    if physics == "elastic":
        s["body_foce"] = [0.1, -0.2, 0.05]
    gl, ol = gpu_loss(etype, physics, m, s), oracle_loss(etype, physics, m, s)
    name = "E" if physics == "elastic" else "K"
    resp = _response(gl, formula, name, gl.GetNumberOfControls())
    ro = fo.ResponseOracle(ol, parse_response_formula(formula, name, "U" if physics == "elastic" else "T",
                                                      gl.number_dofs_per_node))
    rng = np.random.default_rng(72)
    ctrl = 0.5 + rng.random(gl.GetNumberOfControls())
    u = ol.full_dof_vector(0.05 * rng.standard_normal(ol.total_dofs))
    adj = rng.standard_normal(ol.total_dofs)
    v = float(resp.ComputeValue(ctrl, u))
    assert abs(v - ro.value(ctrl, u)) <= TOL * max(1.0, abs(ro.value(ctrl, u)))
    jac, rhs = resp.ComputeAdjointJacobianMatrixAndRHSVector(ctrl, u)
    A, rhs_o = ro.adjoint_jacobian_and_rhs(ctrl, u)
    assert rel_fro(rhs.cpu().numpy(), rhs_o) < TOL
    assert rel_fro(jac.to_scipy().toarray(), A.toarray()) < TOL
    assert rel_fro(resp.ComputeAdjointNodalControlDerivatives(ctrl, u, adj).cpu().numpy(),
                   ro.nodal_control_derivatives(ctrl, u, adj)) < TOL
    assert rel_fro(resp.ComputeAdjointNodalShapeDerivatives(ctrl, u, adj).cpu().numpy(),
                   ro.nodal_shape_derivatives(ctrl, u, adj)) < TOL


def test_adjoint_solver_matches_direct_solve(cuda):
    """AdjointFiniteElementSolver: K^T_BC adjoint = -dJ/du with Jacobi-BiCGSTAB
    against an FP64 direct solve of the oracle's transposed system."""
    from folax_gb300.solvers import AdjointFiniteElementSolver
    m = make_mesh("hex8", 4, seed=73)
    s = {"dirichlet_bc_dict": bc_dict("hex8", "elastic"), "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3}}
    gl, ol = gpu_loss("hex8", "elastic", m, s), oracle_loss("hex8", "elastic", m, s)
    resp = _response(gl, "(E**2)*U[2]", "E", m.GetNumberOfNodes())
    rng = np.random.default_rng(74)
    ctrl = 0.5 + rng.random(m.GetNumberOfNodes())
    u = ol.full_dof_vector(0.01 * rng.standard_normal(ol.total_dofs))
    solver = AdjointFiniteElementSolver("adj", resp, {"linear_solver_settings": {"tol": 1e-9, "maxiter": 5000,
                                                                                "vector_precision": "fp64"}})
    solver.Initialize()
    lam = solver.Solve(ctrl, u, np.zeros(ol.total_dofs)).double().cpu().numpy()
    ro = fo.ResponseOracle(ol, [(1.0, 2, (0, 0, 1))])
    A, rhs = ro.adjoint_jacobian_and_rhs(ctrl, u)
    assert solver.last_linear_info["status"] == 0
    assert rel_fro(lam, fo.direct_solve(A, rhs)) < TOL
