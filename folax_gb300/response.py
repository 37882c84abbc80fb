"""FiniteElementResponse on the device (fol/responses/fe_response.py:17-526).

The reference compiles its response formula string into a JAX function of the
Gauss-point control and dofs (fe_response.py:58-62: ``lambda <control>, <U>:
formula``).  Here the formula is parsed (Python ``ast``, no eval) into a
polynomial -- a list of monomials ``coeff * d**p * u_0**q0 * u_1**q1 *
u_2**q2`` -- which ``folgb_response`` evaluates and differentiates in one
element kernel.  Supported syntax: numbers, the control name, ``U[i]``, unary
``+``/``-``, ``+``, ``-``, ``*``, division by a constant, ``**`` with a
non-negative integer exponent, parentheses.  Anything else (``jnp``
functions, non-polynomial terms) raises ``NotImplementedError``.
"""
from __future__ import annotations

import ast
import ctypes as C

from . import _capi as capi
from .loss import _dev, _torch

MAX_MONOMIALS = 16


class _Poly:
    """Polynomial in d and u_0..u_2: {(p, q0, q1, q2): coeff}."""

    def __init__(self, terms=None):
        self.terms = {k: v for k, v in (terms or {}).items() if v != 0.0}

    @staticmethod
    def const(c):
        return _Poly({(0, 0, 0, 0): float(c)})

    def __add__(self, o):
        t = dict(self.terms)
        for k, v in o.terms.items():
            t[k] = t.get(k, 0.0) + v
        return _Poly(t)

    def __neg__(self):
        return _Poly({k: -v for k, v in self.terms.items()})

    def __mul__(self, o):
        t = {}
        for ka, va in self.terms.items():
            for kb, vb in o.terms.items():
                k = tuple(a + b for a, b in zip(ka, kb))
                t[k] = t.get(k, 0.0) + va * vb
        return _Poly(t)

    def power(self, n):
        out = _Poly.const(1.0)
        for _ in range(n):
            out = out * self
        return out

    def constant_value(self):
        if any(k != (0, 0, 0, 0) for k in self.terms):
            return None
        return self.terms.get((0, 0, 0, 0), 0.0)


def parse_response_formula(formula: str, control_name: str, dof_name: str, ndof: int):
    """The reference's response formula -> [(coeff, control_power, (q0, q1, q2)), ...]."""

    def bad(node, why):
        raise NotImplementedError(f"response formula {formula!r}: {why} ({ast.dump(node)[:60]})")

    def walk(node):
        if isinstance(node, ast.Expression):
            return walk(node.body)
        if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)):
            return _Poly.const(node.value)
        if isinstance(node, ast.Name):
            if node.id == control_name:
                return _Poly({(1, 0, 0, 0): 1.0})
            bad(node, f"unknown name {node.id}")
        if isinstance(node, ast.Subscript) and isinstance(node.value, ast.Name) and node.value.id == dof_name:
            idx = node.slice
            if isinstance(idx, ast.Constant) and isinstance(idx.value, int) and 0 <= idx.value < ndof:
                k = [0, 0, 0, 0]
                k[1 + idx.value] = 1
                return _Poly({tuple(k): 1.0})
            bad(node, f"{dof_name}[...] needs a constant index below {ndof}")
        if isinstance(node, ast.UnaryOp) and isinstance(node.op, (ast.UAdd, ast.USub)):
            v = walk(node.operand)
            return -v if isinstance(node.op, ast.USub) else v
        if isinstance(node, ast.BinOp):
            a, b = walk(node.left), walk(node.right)
            if isinstance(node.op, ast.Add):
                return a + b
            if isinstance(node.op, ast.Sub):
                return a + (-b)
            if isinstance(node.op, ast.Mult):
                return a * b
            if isinstance(node.op, ast.Div):
                c = b.constant_value()
                if c is None or c == 0.0:
                    bad(node, "division by a non-constant")
                return a * _Poly.const(1.0 / c)
            if isinstance(node.op, ast.Pow):
                n = b.constant_value()
                if n is None or n < 0 or float(n) != int(n):
                    bad(node, "exponent must be a non-negative integer constant")
                return a.power(int(n))
        bad(node, "unsupported expression")

    poly = walk(ast.parse(formula, mode="eval"))
    monomials = [(v, k[0], (k[1], k[2], k[3])) for k, v in sorted(poly.terms.items())]
    if len(monomials) > MAX_MONOMIALS:
        raise NotImplementedError(f"response formula expands to {len(monomials)} monomials (max {MAX_MONOMIALS})")
    return monomials


class FiniteElementResponse:
    """Same constructor and methods as the reference's FiniteElementResponse
    for thermal and linear-elastic losses; results are CUDA tensors."""

    def __init__(self, name: str, response_formula: str, fe_loss, control):
        self._name = name
        self.response_formula = response_formula
        self.fe_loss = fe_loss
        self.control = control
        self.initialized = False

    def GetName(self):
        return self._name

    def Initialize(self, reinitialize=False):
        if self.initialized and not reinitialize:
            return
        self.fe_loss.Initialize()
        self.control.Initialize()
        dof_name = self.fe_loss.dofs[0][0]
        self.monomials = parse_response_formula(self.response_formula, self.control.GetName(), dof_name,
                                                self.fe_loss.number_dofs_per_node)
        arr = (capi.Monomial * max(1, len(self.monomials)))()
        for i, (c, p, q) in enumerate(self.monomials):
            arr[i].coeff = c
            arr[i].control_power = p
            for j in range(3):
                arr[i].dof_power[j] = q[j]
        self._mono = arr
        plan = self.fe_loss._plan
        n = int(plan.lib.folgb_response_workspace_bytes(plan.handle))
        torch = _torch()
        self._ws = torch.empty(max(n, 256), dtype=torch.uint8, device="cuda")
        self.initialized = True

    def _call(self, control, dofs, adjoint=None, value=False, rhs=False, dcontrol=False, dxyz=False):
        torch = _torch()
        plan = self.fe_loss._plan
        c = _dev(control).reshape(-1)
        u = _dev(dofs).reshape(-1)
        a = _dev(adjoint).reshape(-1) if adjoint is not None else None
        out_v = torch.empty(1, dtype=torch.float32, device="cuda") if value else None
        out_r = torch.empty_like(u) if rhs else None
        out_c = torch.empty_like(c) if dcontrol else None
        out_x = torch.empty(3 * plan.num_nodes, dtype=torch.float32, device="cuda") if dxyz else None
        rc = plan.lib.folgb_response(plan.handle, len(self.monomials), C.cast(self._mono, C.c_void_p), capi.ptr(c),
                                     capi.ptr(u), capi.ptr(a), capi.ptr(out_v), capi.ptr(out_r), capi.ptr(out_c),
                                     capi.ptr(out_x), capi.ptr(self._ws), self._ws.numel(), capi.stream_handle())
        capi.check("folgb_response", rc)
        return out_v, out_r, out_c, out_x

    def ComputeValue(self, nodal_control_values, nodal_dof_values):
        """J (fe_response.py:208-225), a 0-d CUDA tensor."""
        return self._call(nodal_control_values, nodal_dof_values, value=True)[0][0]

    def ComputeAdjointJacobianMatrixAndRHSVector(self, nodal_control_values, nodal_dof_values):
        """(transposed BC Jacobian, -(dJ/du) with zeros on Dirichlet dofs)
        (fe_response.py:244-283)."""
        rhs = self._call(nodal_control_values, nodal_dof_values, rhs=True)[1]
        jac, _ = self.fe_loss.ComputeJacobianMatrixAndResidualVector(nodal_control_values, nodal_dof_values,
                                                                     transpose_jacobian=True)
        return jac, rhs

    def ComputeAdjointNodalControlDerivatives(self, nodal_control_values, nodal_dof_values, nodal_adj_dof_values):
        """dJ/dcontrol + adjoint . dR/dcontrol (fe_response.py:486-526)."""
        return self._call(nodal_control_values, nodal_dof_values, nodal_adj_dof_values, dcontrol=True)[2]

    def ComputeAdjointNodalShapeDerivatives(self, nodal_control_values, nodal_dof_values, nodal_adj_dof_values):
        """dJ/dxyz + adjoint . dR/dxyz, [3 N] (fe_response.py:365-406)."""
        return self._call(nodal_control_values, nodal_dof_values, nodal_adj_dof_values, dxyz=True)[3]

    def Finalize(self):
        pass
