"""Tetrahedra in patches of six (k_tet_patch + the patch-record gather)
against the per-element path (element kernel + gather, kernel_variant
"generic") and the FP64 oracles.

Meshes: the 6-tet split of jittered hexahedral grids (every 6 consecutive tets
on 8 nodes), its nodes renumbered at random plus nodes no element uses (the
patches do not depend on the node numbering), and the same tets in a random
element order (no patches: the per-element path runs).  Inputs: element or
nodal controls in [0.5, 1.5), dofs = 0.05 z + N(0, (0.05 h)^2) (no inverted
element: the neo-Hookean energies need J > 0), batch 3, loss exponents 1 and
2 (1.5 where the energy cannot be negative).  Tolerances: 1e-5 relative
(Frobenius) against the oracle; the two GPU paths add the same element
results in another order, 1e-6 relative."""
import numpy as np
import pytest

from gpu_cases import bc_dict, c_oracle_loss, gpu_loss, make_mesh, oracle_loss, rel_fro

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _reordered(m, seed, how):
    rng = np.random.default_rng(seed)
    X, T = m.nodes_coordinates, m.elements_nodes["tetra"]
    if how == "nodes":
        N = len(X)
        perm = rng.permutation(N)  # new id -> old id
        inv = np.empty(N, dtype=np.int64)
        inv[perm] = np.arange(N)
        m.nodes_coordinates = np.concatenate([X[perm], 0.5 + 0.01 * rng.standard_normal((3, 3))])
        m.elements_nodes = {"tetra": inv[T]}
        m.node_sets = {k: np.sort(inv[np.asarray(v)]) for k, v in m.node_sets.items()}
        m.node_ids = np.arange(len(m.nodes_coordinates))
    else:  # elements in a random order: no group of 6 stays on 8 nodes
        m.elements_nodes = {"tetra": T[rng.permutation(len(T))]}
    return m


def _settings(layout, exponent=1.0):
    return {"dirichlet_bc_dict": bc_dict("tet4", "elastic"),
            "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3}, "control_layout": layout,
            "loss_function_exponent": exponent}


def _inputs(loss, m, B, seed):
    rng = np.random.default_rng(seed)
    ctrl = 0.5 + rng.random((B, loss.GetNumberOfControls()))
    X = m.nodes_coordinates
    h = 1.0 / round(len(X) ** (1.0 / 3.0))
    u = np.zeros((B, len(X), 3))
    u[:, :, 2] = 0.05 * X[None, :, 2]
    u += 0.05 * h * rng.standard_normal(u.shape)
    return ctrl.astype(np.float32), u.reshape(B, -1).astype(np.float32)


def _run(loss, ctrl, u):
    out = loss.ComputeBatchLossAndGrad(ctrl, u)
    loss.CheckDeviceStatus()
    return [x.cpu().numpy().copy() for x in out[2:]]


@pytest.mark.parametrize("physics", ["neohooke", "elastic", "saint_venant", "neohooke_split"])
@pytest.mark.parametrize("layout", ["element", "nodal"])
@pytest.mark.parametrize("exponent", [1.0, 2.0])
def test_patch_path_matches_per_element_path(cuda, physics, layout, exponent):
    # exponent 2, not 1.5: the neo-Hookean (AD) energy is negative under
    # tension (-mu ln J), and a negative total has no real power 1.5
    m = make_mesh("tet4", 10, seed=71, jitter=0.05)
    s = _settings(layout, exponent)
    patch = gpu_loss("tet4", physics, m, s)
    plain = gpu_loss("tet4", physics, m, {**s, "kernel_variant": "generic"})
    assert patch.KernelFeatures()["tet_patches"]
    ctrl, u = _inputs(patch, m, 3, 72)
    a, b = _run(patch, ctrl, u), _run(plain, ctrl, u)
    for x, y in zip(a, b):
        assert rel_fro(x, y) < 1e-6
    again = _run(patch, ctrl, u)
    for x, y in zip(a, again):
        assert np.array_equal(x, y)  # deterministic


@pytest.mark.parametrize("physics", ["neohooke", "elastic"])
@pytest.mark.parametrize("order", ["split", "nodes", "elements"])
def test_patch_path_against_c_oracle(cuda, physics, order):
    """16^3 split (24,576 tets), batch 3, element controls, against the FP64
    C oracle instance by instance; renumbered nodes keep the patches (the
    unused nodes get zero gradients), shuffled elements lose them."""
    m = make_mesh("tet4", 16, seed=73, jitter=0.05)
    if order != "split":
        m = _reordered(m, 74, order)
    s = _settings("element")
    gl = gpu_loss("tet4", physics, m, s)
    assert gl.KernelFeatures()["tet_patches"] == (order != "elements")
    ctrl, u = _inputs(gl, m, 3, 75)
    losses, du, dc = _run(gl, ctrl, u)
    o = c_oracle_loss("tet4", physics, m, s).batch_loss_and_grads(ctrl.astype(np.float64), u.astype(np.float64))
    for x, z in zip((losses, du, dc), o[2:]):
        assert rel_fro(x, z) < TOL
    if order == "nodes":
        assert np.all(du[:, -9:] == 0.0)


@pytest.mark.parametrize("physics", ["saint_venant", "neohooke_split"])
def test_patch_path_against_python_oracle(cuda, physics):
    m = make_mesh("tet4", 4, seed=76, jitter=0.05)
    s = _settings("nodal", 1.5)
    gl = gpu_loss("tet4", physics, m, s)
    assert gl.KernelFeatures()["tet_patches"]
    ctrl, u = _inputs(gl, m, 2, 77)
    a = _run(gl, ctrl, u)
    o = oracle_loss("tet4", physics, m, s).batch_loss_and_grads(ctrl.astype(np.float64), u.astype(np.float64))
    for x, z in zip(a, o[2:]):
        assert rel_fro(x, z) < TOL
