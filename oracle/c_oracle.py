"""ctypes front end of the C oracle (oracle/fe_oracle_c.c).

TEST INFRASTRUCTURE ONLY: used by tests/ (pinned against the NumPy oracle) and
by bench.py's CPU-baseline and reference legs.  ``CLossOracle`` mirrors
``FELossOracle.batch_loss_and_grads`` (fe_loss.py:250-262 plus its adjoint) for
the thermal, small-strain elastic and neo-Hookean (AD) physics, FP64, OpenMP
over elements; ``assemble_csr`` and ``pcg`` give the FP64 assembled system
(fe_loss.py:264-318) and its Jacobi-CG solution (fe_solver.py:60-78) for the
full-size solve checks.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_c
from .fe_oracle import FELossOracle, gauss_rule

_ET = {"quad4": 0, "hex8": 1, "tet4": 2}
_PH = {"thermal": 0, "elastic": 1, "neohooke": 2}
_lib = None


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build_c.build())
        P = C.c_void_p
        lib.feo_loss_adjoint.restype = C.c_int
        lib.feo_loss_adjoint.argtypes = [C.c_int, C.c_int, C.c_int, P, P, C.c_int, C.c_double, C.c_double, P,
                                         C.c_double, C.c_double, C.c_int64, P, C.c_int64, P, P, P, P, P, P, P, P,
                                         P, P, P, P, C.c_int]
        lib.feo_assemble_csr.restype = C.c_int
        lib.feo_assemble_csr.argtypes = [C.c_int, C.c_int, C.c_int, P, P, C.c_int, C.c_double, C.c_double, P,
                                         C.c_double, C.c_double, C.c_int64, P, C.c_int64, P, P, P, P, P, P, P, P,
                                         C.c_int]
        lib.feo_pcg.restype = C.c_int64
        lib.feo_pcg.argtypes = [C.c_int64, P, P, P, P, P, C.c_double, C.c_int64, P, P, C.c_int]
        lib.feo_max_threads.restype = C.c_int
        lib.feo_max_threads.argtypes = []
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data if a is not None else None


def pcg(indptr, indices, values, b, rtol=1e-12, maxiter=100000, threads=0):
    """FP64 Jacobi-preconditioned CG (x0 = 0) on a CSR matrix with int32
    pattern; stops on the true residual.  Returns (x, iterations, relative
    residual)."""
    lib = load()
    ip = np.ascontiguousarray(indptr, dtype=np.int32)
    ix = np.ascontiguousarray(indices, dtype=np.int32)
    v = np.ascontiguousarray(values, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    n = len(ip) - 1
    x = np.empty(n)
    work = np.empty(5 * n)
    rel = C.c_double()
    it = lib.feo_pcg(n, _p(ip), _p(ix), _p(v), _p(bb), _p(x), float(rtol), int(maxiter), C.byref(rel), _p(work),
                     int(threads))
    if it < 0:
        raise ValueError("feo_pcg: bad arguments")
    return x, int(it), rel.value


class CLossOracle:
    """Same constructor arguments as FELossOracle (thermal / elastic / neo-Hooke)."""

    def __init__(self, *args, threads: int = 0, **kw):
        self.py = FELossOracle(*args, **kw)
        o = self.py
        if o.physics not in _PH:
            raise ValueError(f"C oracle covers thermal, elastic and neohooke, not {o.physics}")
        self.lib = load()
        self.threads = int(threads)
        pts, wts = gauss_rule(o.etype, o.num_gp)
        self.gp = np.ascontiguousarray(pts, dtype=np.float64)
        self.gw = np.ascontiguousarray(wts, dtype=np.float64)
        self.conn = np.ascontiguousarray(o.conn, dtype=np.int64)
        x3 = np.zeros((o.num_nodes, 3))
        x3[:, : o.xyz.shape[1]] = o.xyz
        self.xyz = np.ascontiguousarray(x3)
        slots = self.conn.ravel()
        order = np.argsort(slots, kind="stable")
        self.inc_slot = np.ascontiguousarray(order, dtype=np.int64)
        self.inc_ptr = np.zeros(o.num_nodes + 1, dtype=np.int64)
        np.cumsum(np.bincount(slots, minlength=o.num_nodes), out=self.inc_ptr[1:])
        self.dmask = np.zeros(o.total_dofs, dtype=np.uint8)
        self.dmask[o.dirichlet_indices] = 1
        bf = np.zeros(3)
        if o.body_force is not None and o.physics == "elastic":
            b = np.asarray(o.body_force, dtype=np.float64).ravel()[: o.dim]
            bf[: len(b)] = b
        self.bf = bf
        E = len(self.conn)
        self.rec = np.empty(E * o.nen * o.ndof)
        self.gde = np.empty(E * o.nen)
        self.en = np.empty(E)

    @property
    def max_threads(self) -> int:
        return int(self.lib.feo_max_threads())

    def loss_adjoint(self, ctrl, u_full):
        """Total energy, assembled residual (zero on Dirichlet dofs) and
        d energy / d control of one instance; u_full has Dirichlet values set."""
        o = self.py
        ctrl = np.ascontiguousarray(ctrl, dtype=np.float64)
        u = np.ascontiguousarray(u_full, dtype=np.float64)
        du = np.empty(o.total_dofs)
        dc = np.empty_like(ctrl)
        tot = C.c_double()
        layout = 1 if o.control_layout == "element" else 0
        rc = self.lib.feo_loss_adjoint(_ET[o.etype], _PH[o.physics], len(self.gw), _p(self.gp), _p(self.gw), layout,
                                       o.young, o.nu, _p(self.bf), o.beta, o.c, len(self.conn), _p(self.conn),
                                       o.num_nodes, _p(self.xyz), _p(self.inc_ptr), _p(self.inc_slot),
                                       _p(self.dmask), _p(ctrl), _p(u), C.byref(tot), _p(du), _p(dc), _p(self.rec),
                                       _p(self.gde), _p(self.en), self.threads)
        if rc == 1:
            raise ValueError("feo_loss_adjoint: bad arguments")
        return tot.value, du, dc, rc == 2

    def assemble_csr(self, ctrl, u_full, indptr, indices):
        """FP64 BC-applied residual and Jacobian values of one instance in the
        given canonical CSR pattern (thermal / elastic); u_full has the
        Dirichlet values set.  Returns (residual, values)."""
        o = self.py
        ctrl = np.ascontiguousarray(ctrl, dtype=np.float64)
        u = np.ascontiguousarray(u_full, dtype=np.float64)
        ip = np.ascontiguousarray(indptr, dtype=np.int32)
        ix = np.ascontiguousarray(indices, dtype=np.int32)
        res = np.empty(o.total_dofs)
        vals = np.empty(len(ix))
        layout = 1 if o.control_layout == "element" else 0
        rc = self.lib.feo_assemble_csr(_ET[o.etype], _PH[o.physics], len(self.gw), _p(self.gp), _p(self.gw), layout,
                                       o.young, o.nu, _p(self.bf), o.beta, o.c, len(self.conn), _p(self.conn),
                                       o.num_nodes, _p(self.xyz), _p(self.dmask), _p(ctrl), _p(u), _p(ip), _p(ix),
                                       _p(res), _p(vals), self.threads)
        if rc == 1:
            raise ValueError("feo_assemble_csr: bad arguments or an entry outside the pattern")
        return res, vals

    def batch_loss_and_grads(self, batch_ctrl, batch_u):
        """Same returns as FELossOracle.batch_loss_and_grads."""
        o = self.py
        batch_ctrl = np.atleast_2d(np.asarray(batch_ctrl, dtype=np.float64))
        batch_u = np.atleast_2d(np.asarray(batch_u, dtype=np.float64))
        B = batch_u.shape[0]
        if batch_ctrl.shape[0] == 1 and B > 1:
            batch_ctrl = np.repeat(batch_ctrl, B, axis=0)
        p = o.exponent
        losses = np.zeros(B)
        du = np.zeros_like(batch_u)
        dctrl = np.zeros_like(batch_ctrl)
        for b in range(B):
            tot, g, gc, _ = self.loss_adjoint(batch_ctrl[b], o.full_dof_vector(batch_u[b]))
            losses[b] = tot ** p
            scale = p * tot ** (p - 1.0) / B if p != 1.0 else 1.0 / B
            du[b] = scale * g
            dctrl[b] = scale * gc
        return losses.mean(), (losses.min(), losses.max(), losses.mean()), losses, du, dctrl
