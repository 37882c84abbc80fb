"""Newton with an energy line search on the neo-Hookean (AD) model with the
consistent shear convention (residual = energy gradient): the minimiser of
the loss, which the reference's undamped Newton does not reach beyond small
meshes (its tangent is indefinite near u = 0: S(I) = -mu I).

The device-resident solve (folgb_newton, line_search = 1) is checked against
the FP64 oracle's line-search Newton (direct solves), against the host-driven
loop with the same rule, and by the fused loss gradient at the root."""
import numpy as np
import pytest

from gpu_cases import gpu_loss, oracle_loss, rel_fro
from folax_gb300 import workloads

pytestmark = pytest.mark.gpu


def _problem(n, seed=2024):
    mesh, settings, E, _ = workloads.neohooke_tets(n, 1, seed)
    settings = dict(settings, voigt_shear_mode="consistent")
    return mesh, settings, E[0]


def _solver(loss, resident, abs_tol):
    from folax_gb300.solvers import FiniteElementNonLinearResidualBasedSolver
    s = FiniteElementNonLinearResidualBasedSolver("nl", loss, {
        "linear_solver_settings": {"solver": "JAX-bicgstab", "tol": 1e-8, "maxiter": 20000, "vector_precision": "fp64"},
        "nonlinear_solver_settings": {"load_incr": 5, "maxiter": 60, "abs_tol": abs_tol, "rel_tol": 1e-10,
                                      "device_resident": resident, "line_search": True}})
    s.Initialize()
    return s


@pytest.mark.parametrize("n", [4, 6])
def test_line_search_newton_reaches_the_oracle_minimiser(cuda, n):
    from oracle import fe_oracle as fo
    mesh, settings, E = _problem(n)
    gl = gpu_loss("tet4", "neohooke", mesh, settings)
    solver = _solver(gl, True, 1e-6)
    u = solver.Solve(E, np.zeros(gl.GetTotalNumberOfDOFs(), dtype=np.float32)).double().cpu().numpy()
    gl.CheckDeviceStatus()
    info = solver.last_newton_info
    assert info["status"] == 0 and solver.history[-1]["res_norm"] < 1e-6
    ol = oracle_loss("tet4", "neohooke", mesh, settings)
    u_ref, hist = fo.newton_solve(ol, E.astype(np.float64), np.zeros(ol.total_dofs), load_incr=5, maxiter=60,
                                  abs_tol=1e-10, rel_tol=1e-12, line_search=True)
    assert hist[-1][2] < 1e-9
    assert rel_fro(u, u_ref) < 1e-4
    # the root is a minimiser of the loss: its fused gradient vanishes
    _, _, _, du0, _ = gl.ComputeBatchLossAndGrad(E[None], np.zeros((1, gl.GetTotalNumberOfDOFs())))
    _, _, _, du, _ = gl.ComputeBatchLossAndGrad(E[None], u[None])
    assert float(du.norm()) < 1e-4 * float(du0.norm())


def test_device_and_host_line_search_agree(cuda):
    mesh, settings, E = _problem(4, seed=7)
    gl = gpu_loss("tet4", "neohooke", mesh, settings)
    u0 = np.zeros(gl.GetTotalNumberOfDOFs(), dtype=np.float32)
    a = _solver(gl, True, 1e-6)
    ua = a.Solve(E, u0).double().cpu().numpy()
    b = _solver(gl, False, 1e-6)
    ub = b.Solve(E, u0).double().cpu().numpy()
    assert rel_fro(ua, ub) < 1e-5
    assert a.history[-1]["res_norm"] < 1e-6 and b.history[-1]["res_norm"] < 1e-6


def test_line_search_refuses_an_exponent(cuda):
    from folax_gb300 import _capi
    mesh, settings, E = _problem(2)
    gl = gpu_loss("tet4", "neohooke", mesh, dict(settings, loss_function_exponent=2.0))
    solver = _solver(gl, True, 1e-6)
    with pytest.raises(_capi.FolgbError):
        solver.Solve(E, np.zeros(gl.GetTotalNumberOfDOFs(), dtype=np.float32))
