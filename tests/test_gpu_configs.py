"""Parity at the configured sizes the benchmark reports, against FP64 oracles.

* 64^3 hex8 two-phase elasticity, CSR assembly + Jacobi-PCG: the solution
  at rtol 1e-8 against FP64 Jacobi-CG (C oracle) of the same assembled
  system at the same rtol (bound 1e-6); the solutions at rtol 1e-8 and 1e-9
  against the converged FP64 CG (the truncation error of the stopping rule;
  bound 1e-6 at rtol 1e-9); and against the FP64 solution of the
  FP64-assembled system (the whole fp32 pipeline).  That last error is set by
  storing the matrix in fp32: it is compared with the error of an FP64 solve
  whose only approximation is the FP64 matrix rounded to fp32.
* 50 x 50 quad4 heat conduction (the small plain-method configuration): the
  fp32 solve against an FP64 direct solve of the same system (bound 1e-6),
  and against FP64 assembly + direct solve, compared with the floor of
  storing the FP64 matrix in fp32.
* 6-tet split of 64^3 (1,572,864 tets), neo-Hookean, batch 16: losses and
  both gradients of two instances against the C oracle (1e-5).
* 512 uneven quad4 thermal instances (the benchmark's seed): losses and both
  gradients of every instance against the C oracle (1e-5).
The FP64 oracle errors measured here are printed (pytest -s shows them)."""
import numpy as np
import pytest

from gpu_cases import c_oracle_loss, gpu_loss, rel_fro
from folax_gb300 import workloads

pytestmark = pytest.mark.gpu
TOL = 1e-5


def test_c1_pcg_64cubed_solution_against_fp64(cuda):
    torch = cuda
    from folax_gb300.loss import MechanicalLoss3DHexa
    from folax_gb300.solvers import FiniteElementLinearResidualBasedSolver
    from oracle import c_oracle
    mesh, settings, E, _ = workloads.hex8_elastic(64, 2024)
    loss = MechanicalLoss3DHexa("c1", dict(settings), mesh)
    loss.Initialize()
    u0 = loss.ApplyDirichletBCOnDofVector(torch.zeros(loss.GetTotalNumberOfDOFs(), device="cuda"))
    ctrl = torch.tensor(E, device="cuda")
    jac, r = loss.ComputeJacobianMatrixAndResidualVector(ctrl, u0)
    dx = {}
    for rtol in (1e-8, 1e-9):
        solver = FiniteElementLinearResidualBasedSolver("c1", loss, {"linear_solver_settings": {
            "solver": "GB300-pcg", "tol": rtol, "maxiter": 20000, "check_every": 64}})
        solver.Initialize()
        dx[rtol] = solver.LinearSolve(jac, r).double().cpu().numpy()
        assert solver.last_linear_info["status"] == 0
        assert solver.last_linear_info["relative_residual"] <= rtol
    loss.CheckDeviceStatus()
    indptr, indices = jac.indptr.cpu().numpy(), jac.indices.cpu().numpy()
    A32 = jac.data.double().cpu().numpy()
    r32 = r.double().cpu().numpy()
    # the oracle of the solve: FP64 Jacobi-CG (x0 = 0) of the same assembled
    # system at the same tolerance, and converged (rtol 1e-12)
    x_same, _, rel_same = c_oracle.pcg(indptr, indices, A32, -r32, rtol=1e-8)
    x_a, _, rel_a = c_oracle.pcg(indptr, indices, A32, -r32, rtol=1e-12)
    assert rel_same <= 1e-8 and rel_a <= 1e-12
    err_same = rel_fro(dx[1e-8], x_same)
    err_conv = {t: rel_fro(dx[t], x_a) for t in dx}
    # the pipeline: FP64 assembly + FP64 CG, and the fp32-rounding floor
    cl = c_oracle_loss("hex8", "elastic", mesh, settings)
    u_full = cl.py.full_dof_vector(np.zeros(cl.py.total_dofs))
    R64, V64 = cl.assemble_csr(E.astype(np.float64), u_full, indptr, indices)
    assert rel_fro(r32, R64) < TOL and rel_fro(A32, V64) < TOL
    x_b, _, rel_b = c_oracle.pcg(indptr, indices, V64, -R64, rtol=1e-12)
    assert rel_b <= 1e-12
    x_c, _, _ = c_oracle.pcg(indptr, indices, V64.astype(np.float32).astype(np.float64), -R64, rtol=1e-12)
    err_pipeline = rel_fro(dx[1e-9], x_b)
    err_floor = rel_fro(x_c, x_b)
    print(f"\nC1 64^3 PCG: rtol 1e-8 vs FP64 CG at rtol 1e-8 {err_same:.3e}, vs converged FP64 CG "
          f"{err_conv[1e-8]:.3e}; rtol 1e-9 vs converged {err_conv[1e-9]:.3e}; vs the FP64 pipeline "
          f"{err_pipeline:.3e}; fp32-rounded FP64 matrix alone {err_floor:.3e}")
    assert err_same <= 1e-6
    assert err_conv[1e-9] <= 1e-6
    assert err_pipeline <= 2.0 * err_floor + 1e-6


def test_c0_thermal_50_solve_against_fp64_pipeline(cuda):
    """Plain method, small: the 50 x 50 quad4 heat conduction solve through
    the solver API (fp32 assembly, PCG to rtol 1e-10 with fp64 dots and
    iterate) against the FP64 pipeline the configuration names (FP64
    assembly and a direct solve), and the assembled system against the FP64
    assembly."""
    torch = cuda
    from folax_gb300.loss import ThermalLoss2DQuad
    from folax_gb300.solvers import FiniteElementLinearResidualBasedSolver
    from oracle import fe_oracle as fo
    m, settings, k = workloads.square_thermal(50, 5)
    loss = ThermalLoss2DQuad("c0", dict(settings), m)
    loss.Initialize()
    solver = FiniteElementLinearResidualBasedSolver("c0", loss, {"linear_solver_settings": {
        "solver": "GB300-pcg", "tol": 1e-10, "maxiter": 20000, "vector_precision": "fp32"}})
    solver.Initialize()
    T = solver.Solve(torch.tensor(k, dtype=torch.float32, device="cuda"),
                     torch.zeros(loss.GetTotalNumberOfDOFs(), device="cuda")).double().cpu().numpy()
    assert solver.last_linear_info["status"] == 0
    ol = fo.FELossOracle("quad4", "thermal", m.nodes_coordinates, m.elements_nodes["quad"],
                         dirichlet=settings["dirichlet_bc_dict"], node_sets=m.node_sets, num_gp=2,
                         control_layout="element")
    T_ref = fo.linear_solve(ol, k, np.zeros(ol.total_dofs))
    u0 = loss.ApplyDirichletBCOnDofVector(torch.zeros(loss.GetTotalNumberOfDOFs(), device="cuda"))
    jac, r = loss.ComputeJacobianMatrixAndResidualVector(torch.tensor(k, dtype=torch.float32, device="cuda"), u0)
    A, R = ol.csr(k, ol.full_dof_vector(np.zeros(ol.total_dofs)))
    # the solver: the GPU solve against an FP64 direct solve of the same fp32 system
    A32 = jac.to_scipy().astype(np.float64)
    T_same = u0.double().cpu().numpy() + fo.direct_solve(A32, -r.double().cpu().numpy())
    # the floor of storing the matrix in fp32: the FP64 matrix rounded to fp32
    A_rounded = A.copy()
    A_rounded.data = A_rounded.data.astype(np.float32).astype(np.float64)
    u_full = ol.full_dof_vector(np.zeros(ol.total_dofs))
    T_floor = u_full + fo.direct_solve(A_rounded, -R)
    err_T, err_A = rel_fro(T, T_ref), rel_fro(jac.data.cpu().numpy(), A.data)
    err_solver, err_floor = rel_fro(T, T_same), rel_fro(T_floor, T_ref)
    print(f"\nC0 50^2: solution vs the same fp32 system solved in FP64 {err_solver:.3e}; vs FP64 assembly + "
          f"direct solve {err_T:.3e}; fp32-rounded FP64 matrix alone {err_floor:.3e}; CSR values vs FP64 "
          f"{err_A:.3e}")
    assert err_A < TOL
    assert err_solver < 1e-6
    assert err_T <= 2.0 * err_floor + 1e-6


def test_c4_neohooke_64cubed_batch16_against_c_oracle(cuda):
    from folax_gb300.loss import NeoHookeMechanicalLoss3DTetra
    mesh, settings, E, U = workloads.neohooke_tets(64, 16, 2024)
    loss = NeoHookeMechanicalLoss3DTetra("c4", dict(settings), mesh)
    loss.Initialize()
    _, _, losses, du, dE = loss.ComputeBatchLossAndGrad(E, U)
    loss.CheckDeviceStatus()
    losses, du, dE = losses.cpu().numpy(), du.cpu().numpy(), dE.cpu().numpy()
    cl = c_oracle_loss("tet4", "neohooke", mesh, settings)
    B = len(U)
    for i in (0, 9):
        tot, g, gc, bad = cl.loss_adjoint(E[i].astype(np.float64), cl.py.full_dof_vector(U[i].astype(np.float64)))
        assert not bad
        errs = (rel_fro(losses[i], tot), rel_fro(du[i] * B, g), rel_fro(dE[i] * B, gc))
        print(f"\nC4 instance {i}: loss {errs[0]:.2e}, dL/du {errs[1]:.2e}, dL/dE {errs[2]:.2e}")
        assert max(errs) < TOL, errs


def test_c3_512_instances_against_c_oracle(cuda):
    torch = cuda
    from folax_gb300.batched import BatchedFELoss
    meshes, settings, ks = workloads.thermal_instances(512, 11)
    bl = BatchedFELoss("quad", "thermal", meshes, settings, elements_per_tile=2048)
    ctrl = np.concatenate(ks)
    T = torch.rand(bl.total_dofs, device="cuda", generator=torch.Generator(device="cuda").manual_seed(11))
    _, losses, du, dc = bl.ComputeLossAndGrad(torch.tensor(ctrl, dtype=torch.float32, device="cuda"), T)
    losses, du, dc, T = losses.cpu().numpy(), du.cpu().numpy(), dc.cpu().numpy(), T.cpu().numpy()
    I = len(meshes)
    worst = np.zeros(3)
    for i, m in enumerate(meshes):
        cl = c_oracle_loss("quad4", "thermal", m, settings)
        a, b = bl.dof_offsets[i], bl.dof_offsets[i + 1]
        c0, c1 = bl.control_offsets[i], bl.control_offsets[i + 1]
        tot, g, gc, bad = cl.loss_adjoint(ks[i], cl.py.full_dof_vector(T[a:b].astype(np.float64)))
        assert not bad
        errs = np.array([rel_fro(losses[i], tot), rel_fro(du[a:b] * I, g), rel_fro(dc[c0:c1] * I, gc)])
        worst = np.maximum(worst, errs)
    print(f"\nC3 512 instances, worst over instances: loss {worst[0]:.2e}, dL/dT {worst[1]:.2e}, dL/dk {worst[2]:.2e}")
    assert worst.max() < TOL, worst
