"""FE solvers: the reference's solver API over the GB300 assembly and PCG.

Mirrors fol/solvers/solver.py:11-49, fe_solver.py:21-105,
fe_linear_residual_based_solver.py:10-22 and
fe_nonlinear_residual_based_solver.py:15-170.  The linear solve runs on the
assembled CSR with Jacobi preconditioning, fp64 inner products and norms and
x0 = 0.  The solver name "GB300-pcg" selects CG (folgb_pcg / folgb_krylov);
every other name, the reference's "JAX-bicgstab", "JAX-direct" and
"PETSc-*" choices included, selects BiCGSTAB, which also handles the
nonsymmetric and indefinite tangents the reference's default solver is used
for.  With the row-only Dirichlet rule (fe_loss.py:191-207) the BC rows of the
system are diag * dx = 0, so a Krylov solve started from 0 never leaves the
free-dof subspace: for CG it solves K_FF dx_F = -r_F as a symmetric system.
"""
from __future__ import annotations

import copy
import ctypes as C

import numpy as np

from . import _capi as capi
from .loss import FiniteElementLoss, _dev, _torch


def UpdateDefaultDict(default_dict: dict, given_dict: dict):
    """Only keys already in default_dict are taken (fol/tools/usefull_functions.py:569-573)."""
    out = copy.deepcopy(default_dict)
    out.update({k: given_dict[k] for k in default_dict if k in given_dict})
    return out


class Solver:
    def __init__(self, solver_name: str) -> None:
        self._name = solver_name

    def GetName(self) -> str:
        return self._name

    def Initialize(self) -> None:
        pass

    def Solve(self, control_vars, dofs):
        raise NotImplementedError

    def BatchSolve(self, batch_control_vars, batch_dofs):
        """solver.py:47-49 (a vmap there; a loop of device solves here)."""
        torch = _torch()
        ctrl = _dev(batch_control_vars)
        dofs = _dev(batch_dofs)
        return torch.stack([self.Solve(c, d) for c, d in zip(ctrl, dofs)]).squeeze()

    def Finalize(self) -> None:
        pass


class FiniteElementSolver(Solver):
    def __init__(self, fe_solver_name: str, fe_loss_function: FiniteElementLoss, fe_solver_settings: dict = {}):
        super().__init__(fe_solver_name)
        self.fe_loss_function = fe_loss_function
        self.fe_solver_settings = fe_solver_settings
        self.linear_solver_settings = {"solver": "JAX-bicgstab", "tol": 1e-6, "atol": 1e-6, "maxiter": 1000,
                                       "pre-conditioner": "ilu", "check_every": 32, "vector_precision": "auto"}
        self.last_linear_info = None

    def Initialize(self) -> None:
        if "linear_solver_settings" in self.fe_solver_settings:
            self.linear_solver_settings = UpdateDefaultDict(self.linear_solver_settings,
                                                            self.fe_solver_settings["linear_solver_settings"])
        name = self.linear_solver_settings["solver"]
        known = ["PETSc-bcgsl", "PETSc-tfqmr", "PETSc-minres", "PETSc-gmres", "JAX-direct", "JAX-bicgstab",
                 "GB300-pcg", "GB300-bicgstab"]
        if name not in known:
            raise ValueError(f"linear solver {name} does exist, available options are {known}")
        # CG for the SPD systems it was asked for; every other name keeps the
        # reference's default behaviour (a Krylov method that tolerates
        # nonsymmetric / indefinite tangents): Jacobi-BiCGSTAB.
        self.LinearSolve = self.PCGLinearSolver if name == "GB300-pcg" else self.BiCGSTABLinearSolver

    def _vector_bits(self) -> int:
        """Krylov vector precision: "fp32", "fp64", or "auto" (fp64 for the
        Neo-Hookean tangent, which is indefinite near u = 0 and defeats fp32
        recurrences; fp32 otherwise)."""
        v = self.linear_solver_settings.get("vector_precision", "auto")
        if v == "auto":
            return 64 if getattr(self.fe_loss_function, "physics", None) == capi.NEOHOOKE else 32
        if v not in ("fp32", "fp64"):
            raise ValueError(f"vector_precision must be auto, fp32 or fp64, not {v}")
        return 64 if v == "fp64" else 32

    def _krylov(self, method, tangent_matrix, residual_vector):
        torch = _torch()
        plan = tangent_matrix.plan
        bits = self._vector_bits()
        # fixed right-hand-side and solution buffers per plan: the library
        # caches the instantiated solve graph per set of buffers, so repeated
        # solves on one plan launch the cached graph
        bufs = getattr(self, "_krylov_bufs", None)
        if bufs is None or bufs[0] is not plan:
            n = plan.total_dofs
            bufs = (plan, torch.empty(n, dtype=torch.float32, device="cuda"),
                    torch.empty(n, dtype=torch.float32, device="cuda"))
            self._krylov_bufs = bufs
        _, b, x = bufs
        torch.neg(_dev(residual_vector).reshape(-1), out=b)
        ws = plan.workspace(capi.OP_KRYLOV64 if bits == 64 else capi.OP_PCG)
        iters, rel = C.c_int32(), C.c_double()
        s = self.linear_solver_settings
        rc = plan.lib.folgb_krylov(plan.handle, method, bits, capi.ptr(tangent_matrix.data),
                                   capi.ptr(tangent_matrix.inv_diag), capi.ptr(b), capi.ptr(x), float(s["tol"]),
                                   int(s["maxiter"]), int(s.get("check_every", 32)), C.byref(iters), C.byref(rel),
                                   capi.ptr(ws), ws.numel(), capi.stream_handle())
        name = ("folgb_pcg" if method == capi.KRYLOV_CG else "folgb_bicgstab") + ("" if bits == 32 else "_fp64")
        self.last_linear_info = {"solver": name, "iterations": iters.value, "relative_residual": rel.value,
                                 "status": rc, "vector_bits": bits}
        if rc not in (capi.OK, capi.ERR_NOT_CONVERGED):
            capi.check(name, rc)
        return x.clone()

    def PCGLinearSolver(self, tangent_matrix, residual_vector, dofs_vector=None):
        """Solve tangent_matrix dx = -residual with Jacobi-PCG (x0 = 0); returns dx."""
        return self._krylov(capi.KRYLOV_CG, tangent_matrix, residual_vector)

    def BiCGSTABLinearSolver(self, tangent_matrix, residual_vector, dofs_vector=None):
        """Solve tangent_matrix dx = -residual with Jacobi-BiCGSTAB (x0 = 0); returns dx.
        (fe_solver.py:60-67 passes x0 = current dofs; dx starts from 0 here.)"""
        return self._krylov(capi.KRYLOV_BICGSTAB, tangent_matrix, residual_vector)


class FiniteElementLinearResidualBasedSolver(FiniteElementSolver):
    """fe_linear_residual_based_solver.py:15-22."""

    def Solve(self, current_control_vars, current_dofs):
        loss = self.fe_loss_function
        u = loss.ApplyDirichletBCOnDofVector(current_dofs)
        jac, r = loss.ComputeJacobianMatrixAndResidualVector(current_control_vars, u)
        du = self.LinearSolve(jac, r, u)
        return u + du


class AdjointFiniteElementSolver(FiniteElementSolver):
    """adjoint_fe_solver.py:11-23: solves K^T_BC adjoint = -dJ/du for a
    FiniteElementResponse (folax_gb300.response)."""

    def __init__(self, adj_fe_solver_name: str, fe_response, adj_fe_solver_settings: dict = {}):
        super().__init__(adj_fe_solver_name, fe_response.fe_loss, adj_fe_solver_settings)
        self.fe_response = fe_response

    def Solve(self, current_control_vars, current_dofs, current_adjoint_dofs=None):
        jac, rhs = self.fe_response.ComputeAdjointJacobianMatrixAndRHSVector(current_control_vars, current_dofs)
        # the linear solver negates its right-hand side (adjoint_fe_solver.py:21-22)
        return self.LinearSolve(jac, -rhs, current_adjoint_dofs)


class FiniteElementNonLinearResidualBasedSolver(FiniteElementLinearResidualBasedSolver):
    """Newton-Raphson with load stepping (fe_nonlinear_residual_based_solver.py:76-170).

    Convergence: |r|_2 < abs_tol or |dx|_2 < rel_tol or maxiter (the
    converged step's update is not applied, as in the reference).  Norms are
    fp64 reductions on the device.  nonlinear_solver_settings
    "device_resident" (default True): the whole solve, load steps, Newton
    iterations and Krylov iterations, runs as one CUDA graph (folgb_newton)
    with no host synchronisation until it ends; False: a host loop with one
    host read per Newton iteration.
    "line_search" (default False, the reference's full steps): True takes
    t dx with the backtracking rule of folgb_newton on the element energy
    (for losses whose residual is the energy gradient, e.g. neo-Hooke with
    voigt_shear_mode "consistent"); "line_search_max_halvings" (default 30)."""

    def __init__(self, fe_solver_name, fe_loss_function, fe_solver_settings: dict = {}, history_plot_settings: dict = {}):
        super().__init__(fe_solver_name, fe_loss_function, fe_solver_settings)
        self.nonlinear_solver_settings = {"rel_tol": 1e-8, "abs_tol": 1e-8, "maxiter": 20, "load_incr": 5,
                                          "device_resident": True, "line_search": False,
                                          "line_search_max_halvings": 30}
        self.history = []
        self.last_newton_info = None

    def Initialize(self) -> None:
        super().Initialize()
        if "nonlinear_solver_settings" in self.fe_solver_settings:
            self.nonlinear_solver_settings = UpdateDefaultDict(self.nonlinear_solver_settings,
                                                               self.fe_solver_settings["nonlinear_solver_settings"])

    def _solve_device_resident(self, current_control_vars, current_dofs):
        torch = _torch()
        loss = self.fe_loss_function
        s = self.nonlinear_solver_settings
        ls = self.linear_solver_settings
        plan = loss._get_csr_plan()
        st = capi.NewtonSettings()
        st.load_steps, st.max_iterations = int(s["load_incr"]), int(s["maxiter"])
        st.abs_tol, st.rel_tol = float(s["abs_tol"]), float(s["rel_tol"])
        st.krylov_method = capi.KRYLOV_CG if self.LinearSolve == self.PCGLinearSolver else capi.KRYLOV_BICGSTAB
        st.vector_bits = self._vector_bits()
        st.krylov_rtol, st.krylov_maxiter = float(ls["tol"]), int(ls["maxiter"])
        st.check_every = int(ls.get("check_every", 32))
        st.line_search = 1 if s.get("line_search", False) else 0
        st.line_search_max_halvings = int(s.get("line_search_max_halvings", 30))
        nbytes = plan.lib.folgb_newton_workspace_bytes(plan.handle, C.byref(st))
        ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        u = _dev(current_dofs).clone().reshape(-1)
        ctrl = _dev(current_control_vars).reshape(-1)
        info = capi.NewtonInfo()
        hist = np.zeros((st.load_steps * st.max_iterations, 4))
        rc = plan.lib.folgb_newton(plan.handle, capi.ptr(ctrl), capi.ptr(u), C.byref(st), C.byref(info),
                                   hist.ctypes.data, capi.ptr(loss._status), capi.ptr(ws), nbytes,
                                   capi.stream_handle())
        self.last_newton_info = {"newton_iterations": info.newton_iterations,
                                 "krylov_iterations": info.krylov_iterations,
                                 "res_norm": info.last_res_norm, "delta_norm": info.last_delta_norm,
                                 "krylov_failures": info.krylov_failures, "status": info.status,
                                 "line_search_halvings": info.line_search_halvings}
        self.history = [{"load_step": int(h[0]), "iteration": int(h[1]), "res_norm": float(h[2]),
                         "delta_dofs_norm": float(h[3])} for h in hist[:info.newton_iterations]]
        if rc == capi.ERR_NAN:
            raise ValueError("Residual norm contains NaN values.")
        if rc == capi.ERR_NOT_CONVERGED:
            raise ValueError("Newton line search found no step that decreases the energy.")
        capi.check("folgb_newton", rc)
        return u

    def _line_search(self, control, u, du, r):
        """Host-loop twin of folgb_newton's backtracking rule: returns t."""
        torch = _torch()
        loss = self.fe_loss_function
        s = self.nonlinear_solver_settings
        e0 = float(loss.ComputeTotalEnergy(control, u))
        slope = -torch.dot(r.double(), du.double()).item()  # predicted decrease
        if not np.isfinite(slope) or slope <= 0.0:
            # not a descent direction: the Jacobi-preconditioned steepest descent step
            du.copy_(-r / self._last_diag)
            slope = -torch.dot(r.double(), du.double()).item()
        if 0.0 <= slope <= 1e-6 * abs(e0):
            return 1.0
        t = 1.0
        for _ in range(int(s["line_search_max_halvings"]) + 1):
            et = float(loss.ComputeTotalEnergy(control, u + t * du))
            if np.isfinite(et) and et <= e0 - 1e-4 * t * max(slope, 0.0) + 2e-6 * abs(e0):
                return t
            t *= 0.5
        raise ValueError("Newton line search found no step that decreases the energy.")

    def Solve(self, current_control_vars, current_dofs):
        torch = _torch()
        loss = self.fe_loss_function
        s = self.nonlinear_solver_settings
        if s.get("device_resident", True):
            return self._solve_device_resident(current_control_vars, current_dofs)
        u = _dev(current_dofs).clone()
        n_steps = int(s["load_incr"])
        self.history = []
        for step in range(1, n_steps + 1):
            u = loss.ApplyDirichletBCOnDofVector(u, step / n_steps)
            for it in range(1, int(s["maxiter"]) + 1):
                jac, r = loss.ComputeJacobianMatrixAndResidualVector(current_control_vars, u)
                res_norm = torch.linalg.vector_norm(r.double()).item()
                if not np.isfinite(res_norm):
                    raise ValueError("Residual norm contains NaN values.")
                du = self.LinearSolve(jac, r, u)
                delta_norm = torch.linalg.vector_norm(du.double()).item()
                self.history.append({"load_step": step, "iteration": it, "res_norm": res_norm,
                                     "delta_dofs_norm": delta_norm, "linear": self.last_linear_info})
                if res_norm < s["abs_tol"] or delta_norm < s["rel_tol"] or it == s["maxiter"]:
                    break
                self._last_diag = 1.0 / jac.inv_diag
                t = self._line_search(current_control_vars, u, du, r) if s.get("line_search", False) else 1.0
                u = u + du if t == 1.0 else u + t * du
        return u
