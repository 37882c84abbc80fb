"""The C oracle (timed CPU baseline) against the NumPy oracle (CPU).

The NumPy oracle is pinned on the reference's golden vectors; these cases pin
the C restatement to it on jittered meshes of every element type, both control
layouts, body force, the loss exponent and the thermal nonlinearity, and check
that the result does not depend on the OpenMP thread count.  The FP64 CSR
assembly is checked against the NumPy oracle's canonical CSR, the FP64 CG
against a direct solve."""
import numpy as np
import pytest

from oracle import c_oracle
from test_oracle_props import _small


def _rel(a, b):
    b = np.asarray(b)
    return float(np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300))


def _pair(etype, physics, layout="nodal", exponent=1.0, bf=None, **extra):
    L, ctrl, u = _small(etype, physics, n=3, seed=5, layout=layout, exponent=exponent, bf=bf)
    for k, v in extra.items():
        setattr(L, k, v)
    kw = dict(dirichlet=None, node_sets=None, num_gp=L.num_gp, young=L.young, nu=L.nu, body_force=L.body_force,
              beta=L.beta, c=L.c, exponent=L.exponent, control_layout=L.control_layout)
    Lc = c_oracle.CLossOracle(L.etype, L.physics, L.xyz, L.conn, **kw)
    # share the Dirichlet sets of the NumPy oracle
    Lc.py.dirichlet_indices, Lc.py.dirichlet_values = L.dirichlet_indices, L.dirichlet_values
    Lc.dmask[:] = 0
    Lc.dmask[L.dirichlet_indices] = 1
    return L, Lc, ctrl, u


@pytest.mark.parametrize("etype,physics", [("quad4", "thermal"), ("hex8", "thermal"), ("tet4", "thermal"),
                                           ("quad4", "elastic"), ("hex8", "elastic"), ("tet4", "elastic"),
                                           ("quad4", "neohooke"), ("hex8", "neohooke"), ("tet4", "neohooke")])
@pytest.mark.parametrize("layout", ["nodal", "element"])
def test_c_oracle_matches_numpy(etype, physics, layout):
    L, Lc, ctrl, u = _pair(etype, physics, layout)
    U = np.stack([u, 0.7 * u])
    ref = L.batch_loss_and_grads(ctrl[None], U)
    got = Lc.batch_loss_and_grads(ctrl[None], U)
    assert _rel(got[2], ref[2]) < 1e-12
    assert _rel(got[3], ref[3]) < 1e-12
    assert _rel(got[4], ref[4]) < 1e-12


@pytest.mark.parametrize("etype", ["hex8", "quad4"])
def test_c_oracle_body_force_exponent(etype):
    bf = [0.1, -0.2, 0.3]
    L, Lc, ctrl, u = _pair(etype, "elastic", "element", exponent=2.0, bf=bf)
    ref = L.batch_loss_and_grads(ctrl[None], u[None])
    got = Lc.batch_loss_and_grads(ctrl[None], u[None])
    for i in (2, 3, 4):
        assert _rel(got[i], ref[i]) < 1e-12


def test_c_oracle_thermal_nonlinear():
    L, Lc, ctrl, u = _pair("hex8", "thermal", beta=1.5, c=2.0)
    Lc.py.beta, Lc.py.c = 1.5, 2.0
    ref = L.batch_loss_and_grads(ctrl[None], u[None])
    got = Lc.batch_loss_and_grads(ctrl[None], u[None])
    for i in (2, 3, 4):
        assert _rel(got[i], ref[i]) < 1e-12


def test_c_oracle_thread_count_invariant():
    L, Lc, ctrl, u = _pair("hex8", "elastic")
    uf = L.full_dof_vector(u)
    Lc.threads = 1
    a = Lc.loss_adjoint(ctrl, uf)
    Lc.threads = max(2, Lc.max_threads)
    b = Lc.loss_adjoint(ctrl, uf)
    assert a[0] == b[0]
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


@pytest.mark.parametrize("etype,physics", [("quad4", "thermal"), ("hex8", "elastic"), ("tet4", "elastic"),
                                           ("hex8", "thermal"), ("quad4", "elastic")])
@pytest.mark.parametrize("layout", ["nodal", "element"])
def test_c_oracle_csr_assembly_matches_numpy(etype, physics, layout):
    L, Lc, ctrl, u = _pair(etype, physics, layout)
    uf = L.full_dof_vector(u)
    A, R = L.csr(ctrl, uf)
    res, vals = Lc.assemble_csr(ctrl, uf, A.indptr, A.indices)
    assert _rel(res, R) < 1e-12
    assert _rel(vals, A.data) < 1e-12


def test_c_oracle_pcg_matches_direct_solve():
    import scipy.sparse.linalg as spla
    from oracle import fe_oracle as fo
    L, Lc, ctrl, u = _pair("hex8", "elastic", "element")
    A, R = L.csr(ctrl, L.full_dof_vector(np.zeros_like(u)))
    x_ref = fo.direct_solve(A, -R)
    x, it, rel = c_oracle.pcg(A.indptr, A.indices, A.data, -R, rtol=1e-13)
    assert it > 0 and rel <= 1e-13
    assert _rel(x, x_ref) < 1e-10
    assert np.linalg.norm(A @ x + R) <= 1.0001e-13 * np.linalg.norm(R)
