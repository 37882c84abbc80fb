"""CUDA path (through the C ABI) against the FP64 oracle and the reference's
golden vectors.  Tolerance: 1e-5 relative (Frobenius) for fp32 results."""
import numpy as np
import pytest

from conftest import arr, golden
from folax_gb300.loss import HEX8_VARIANTS
from folax_gb300.mesh import create_3D_box_mesh
from gpu_cases import bc_dict, gpu_loss, make_mesh, oracle_loss, rel_fro
from oracle import fe_oracle as fo

pytestmark = pytest.mark.gpu
TOL = 1e-5

CASES = [("quad4", "thermal", 8), ("hex8", "elastic", 4), ("tet4", "neohooke", 3), ("quad4", "elastic", 8),
         ("hex8", "neohooke", 3), ("tet4", "thermal", 3), ("hex8", "thermal", 4), ("tet4", "elastic", 3),
         ("quad4", "neohooke", 8)]


def _settings(etype, physics, layout="nodal", exponent=1.0, bf=None, shear="reference"):
    s = {"dirichlet_bc_dict": bc_dict(etype, physics), "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3},
         "control_layout": layout, "loss_function_exponent": exponent, "voigt_shear_mode": shear}
    if bf is not None:
        s["body_foce"] = bf
    return s


@pytest.mark.parametrize("kind,etype", [(k, e) for k in ("mechanical_linear", "neohooke_ad")
                                        for e in ("tet4", "hex8", "quad4")])
def test_element_golden_vectors_on_gpu(cuda, kind, etype):
    """tests/unit/test_mechanical_loss.py / test_neo_hooke_mechanical_loss_AD.py
    through the CUDA kernels (ComputeElement on a one-element mesh)."""
    from folax_gb300 import loss as L
    g = golden(kind + ".json")[etype]
    X = arr(g["xyz"])
    nen, dim = fo.ELEMENTS[etype]
    mesh = make_mesh(etype, 1)
    bf = arr(g["body_force"]).ravel().tolist()
    settings = {"dirichlet_bc_dict": {}, "material_dict": {"young_modulus": 1, "poisson_ratio": 0.3}, "body_foce": bf}
    cls = {("mechanical_linear", "tet4"): L.MechanicalLoss3DTetra, ("mechanical_linear", "hex8"): L.MechanicalLoss3DHexa,
           ("mechanical_linear", "quad4"): L.MechanicalLoss2DQuad, ("neohooke_ad", "tet4"): L.NeoHookeMechanicalLoss3DTetra,
           ("neohooke_ad", "hex8"): L.NeoHookeMechanicalLoss3DHexa, ("neohooke_ad", "quad4"): L.NeoHookeMechanicalLoss2DQuad}[(kind, etype)]
    loss = cls("golden", settings, mesh)
    loss.Initialize()
    en, re, K = loss.ComputeElement(X, np.ones(nen), np.ones(nen * dim))
    np.testing.assert_allclose(K, arr(g["stiffness"]), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(re, arr(g["residual"]), rtol=1e-4 if (etype == "tet4" and kind == "mechanical_linear") else 1e-5,
                               atol=1e-6)


@pytest.mark.parametrize("etype,physics,n", CASES)
@pytest.mark.parametrize("layout", ["nodal", "element"])
def test_loss_adjoint_matches_oracle(cuda, etype, physics, n, layout):
    torch = cuda
    m = make_mesh(etype, n, seed=1)
    s = _settings(etype, physics, layout)
    gl, ol = gpu_loss(etype, physics, m, s), oracle_loss(etype, physics, m, s)
    rng = np.random.default_rng(2)
    B = 2
    nctrl = gl.GetNumberOfControls()
    ctrl = 0.5 + rng.random((B, nctrl))
    # displacement noise scaled to the element size: strains of a few percent
    u = (0.03 / n) * rng.standard_normal((B, gl.GetTotalNumberOfDOFs()))
    mean, (mn, mx, _), losses, du, dc = gl.ComputeBatchLossAndGrad(ctrl, u)
    gl.CheckDeviceStatus()
    omean, _, olosses, odu, odc = ol.batch_loss_and_grads(ctrl, u)
    assert rel_fro(losses.cpu().numpy(), olosses) < TOL
    assert rel_fro(du.cpu().numpy(), odu) < TOL
    assert rel_fro(dc.cpu().numpy(), odc) < TOL
    assert np.all(du.cpu().numpy()[:, ol.dirichlet_indices] == 0)


@pytest.mark.parametrize("layout", ["nodal", "element"])
@pytest.mark.parametrize("bf", [None, [0.3, -0.2, 0.1]])
def test_hex8_sum_factorised_matches_generic_and_oracle(cuda, layout, bf):
    """The sum-factorised hex8 kernel and the generic Gauss loop agree with
    each other and with the oracle (loss, both gradients, residual)."""
    m = make_mesh("hex8", 5, seed=21, jitter=0.15)
    s = _settings("hex8", "elastic", layout, 1.0, bf)
    fast = gpu_loss("hex8", "elastic", m, s)
    generic = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": "generic"})
    ol = oracle_loss("hex8", "elastic", m, s)
    rng = np.random.default_rng(22)
    ctrl = 0.5 + rng.random((2, fast.GetNumberOfControls()))
    u = 0.01 * rng.standard_normal((2, fast.GetTotalNumberOfDOFs()))
    a = fast.ComputeBatchLossAndGrad(ctrl, u)
    g = generic.ComputeBatchLossAndGrad(ctrl, u)
    o = ol.batch_loss_and_grads(ctrl, u)
    for x, y, z in zip(a[2:], g[2:], o[2:]):
        assert rel_fro(x.cpu().numpy(), z) < TOL
        assert rel_fro(y.cpu().numpy(), z) < TOL
    uf = ol.full_dof_vector(u[0])
    _, Rf = fast.ComputeJacobianMatrixAndResidualVector(ctrl[0], uf, with_matrix=False)
    _, Ro = ol.csr(ctrl[0], uf)
    assert rel_fro(Rf.cpu().numpy(), Ro) < TOL


def _hex8_mesh(kind):
    """jittered: every element distorted; box: every element a cube (the
    affine path of the paired kernels); mixed: cubes where x < 0.5, distorted
    elsewhere, so warps hold both kinds."""
    if kind == "jittered":
        return make_mesh("hex8", 4, seed=23, jitter=0.15)
    m = make_mesh("hex8", 4, seed=23, jitter=0.0)
    if kind == "mixed":
        rng = np.random.default_rng(25)
        X = m.nodes_coordinates
        moved = X[:, 0] > 0.6
        X[moved] += (0.15 / 4) * rng.standard_normal((int(moved.sum()), 3))
    return m


@pytest.mark.parametrize("variant", list(range(HEX8_VARIANTS)))
@pytest.mark.parametrize("layout", ["nodal", "element"])
@pytest.mark.parametrize("mesh_kind", ["jittered", "box", "mixed"])
def test_hex8_every_variant_matches_oracle(cuda, variant, layout, mesh_kind):
    """Each autotuner candidate (block size x accumulation scheme) is exact,
    on distorted, affine and mixed meshes."""
    m = _hex8_mesh(mesh_kind)
    s = _settings("hex8", "elastic", layout, 1.0, [0.2, 0.0, -0.1])
    gl = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": variant})
    ol = oracle_loss("hex8", "elastic", m, s)
    rng = np.random.default_rng(24)
    ctrl = 0.5 + rng.random((3, gl.GetNumberOfControls()))
    u = 0.01 * rng.standard_normal((3, gl.GetTotalNumberOfDOFs()))
    a = gl.ComputeBatchLossAndGrad(ctrl, u)
    o = ol.batch_loss_and_grads(ctrl, u)
    for x, z in zip(a[2:], o[2:]):
        assert rel_fro(x.cpu().numpy(), z) < TOL


def _renumbered(m, seed, isolated=2):
    """The same mesh with its nodes and elements in a random order and
    `isolated` extra nodes that no element uses (their gradients must be 0)."""
    rng = np.random.default_rng(seed)
    X = m.nodes_coordinates
    N = len(X)
    perm = rng.permutation(N)          # new id -> old id
    inv = np.empty(N, dtype=np.int64)
    inv[perm] = np.arange(N)
    conn = m.elements_nodes["hexahedron"]
    conn = inv[conn][rng.permutation(len(conn))]
    m.nodes_coordinates = np.concatenate([X[perm], 0.5 + 0.01 * rng.standard_normal((isolated, 3))])
    m.elements_nodes = {"hexahedron": conn}
    m.node_sets = {k: np.sort(inv[np.asarray(v)]) for k, v in m.node_sets.items()}
    m.node_ids = np.arange(len(m.nodes_coordinates))
    return m


@pytest.mark.parametrize("variant", [18, 19])
@pytest.mark.parametrize("layout", ["nodal", "element"])
@pytest.mark.parametrize("exponent,bf", [(1.0, None), (1.5, [0.2, 0.0, -0.1])])
@pytest.mark.parametrize("order", ["structured", "renumbered"])
def test_hex8_tile_kernel_many_tiles(cuda, variant, layout, exponent, bf, order):
    """The tile-local kernel over many tiles (12^3 jittered hex mesh: about
    14 tiles of up to 128 elements, most nodes shared by several tiles), in
    the mesh's own order and with nodes and elements renumbered at random
    plus two nodes no element uses; the loss exponent 1.5 takes the deferred
    scaling path."""
    m = make_mesh("hex8", 12, seed=41, jitter=0.1)
    if order == "renumbered":
        m = _renumbered(m, seed=42)
    s = _settings("hex8", "elastic", layout, exponent, bf)
    gl = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": variant})
    ol = oracle_loss("hex8", "elastic", m, s)
    rng = np.random.default_rng(43)
    ctrl = 0.5 + rng.random((3, gl.GetNumberOfControls()))
    u = 0.004 * rng.standard_normal((3, gl.GetTotalNumberOfDOFs()))
    a = gl.ComputeBatchLossAndGrad(ctrl, u)
    gl.CheckDeviceStatus()
    o = ol.batch_loss_and_grads(ctrl, u)
    for x, z in zip(a[2:], o[2:]):
        assert rel_fro(x.cpu().numpy(), z) < TOL
    if order == "renumbered":
        du = a[3].cpu().numpy()
        assert np.all(du[:, -6:] == 0.0)
        if layout == "nodal":
            assert np.all(a[4].cpu().numpy()[:, -2:] == 0.0)
    b = gl.ComputeBatchLossAndGrad(ctrl, u)
    for x, y in zip(a[2:], b[2:]):
        assert np.array_equal(x.cpu().numpy(), y.cpu().numpy())


def _star_mesh():
    """Hexahedra around an irregular edge: a pentagon split into 5 quads
    (centre, edge midpoints, corners), extruded in two layers; the centre
    node of the middle layer belongs to 10 hexahedra, so a tile holds more
    than 8 of its records (a second local entry)."""
    from folax_gb300.mesh import Mesh
    ang = np.deg2rad(72.0) * np.arange(5)
    corners = np.stack([np.cos(ang), np.sin(ang)], 1)
    mids = 0.5 * (corners + np.roll(corners, -1, axis=0))
    pts2 = np.concatenate([[[0.0, 0.0]], mids, corners])  # 0 centre, 1..5 mids, 6..10 corners
    quads = [(0, 1 + (i - 1) % 5, 6 + i, 1 + i) for i in range(5)]
    zs = [0.0, 0.5, 1.0]
    xyz = np.concatenate([np.column_stack([pts2, np.full(len(pts2), z)]) for z in zs])
    hexes = [[c + 11 * k for c in quad] + [c + 11 * (k + 1) for c in quad] for k in range(2) for quad in quads]
    m = Mesh("star", "star.mem")
    m.nodes_coordinates = xyz
    m.node_ids = np.arange(len(xyz))
    m.elements_nodes = {"hexahedron": np.asarray(hexes, dtype=np.int64)}
    m.node_sets = {"bottom": np.arange(11), "top": np.arange(22, 33)}
    return m


@pytest.mark.parametrize("variant", [18, 19])
@pytest.mark.parametrize("layout", ["nodal", "element"])
def test_hex8_tile_kernel_irregular_edge(cuda, variant, layout):
    m = _star_mesh()
    s = _settings("hex8", "elastic", layout, 1.0, [0.1, 0.0, 0.2])
    gl = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": variant})
    ol = oracle_loss("hex8", "elastic", m, s)
    rng = np.random.default_rng(44)
    ctrl = 0.5 + rng.random((2, gl.GetNumberOfControls()))
    u = 0.01 * rng.standard_normal((2, gl.GetTotalNumberOfDOFs()))
    a = gl.ComputeBatchLossAndGrad(ctrl, u)
    gl.CheckDeviceStatus()
    o = ol.batch_loss_and_grads(ctrl, u)
    for x, z in zip(a[2:], o[2:]):
        assert rel_fro(x.cpu().numpy(), z) < TOL


def _box_mesh(order="structured"):
    """8 x 4 x 6 elements, each the box 0.25 x 0.125 x 0.1875 (dyadic edges:
    every element has exactly the same fp32 Jacobian)."""
    m = create_3D_box_mesh(8, 4, 6, Lx=2.0, Ly=0.5, Lz=1.125)
    return _renumbered(m, seed=46) if order == "renumbered" else m


@pytest.mark.parametrize("variant", [20, 21, 22, 23, 24])
@pytest.mark.parametrize("exponent", [1.0, 1.5])
@pytest.mark.parametrize("order", ["structured", "renumbered"])
def test_hex8_box_kernels_match_oracle(cuda, variant, exponent, order):
    """The uniform-box kernels (element matrix as eight 3 x 3 blocks in the
    Hadamard basis) on a mesh of identical non-cubic boxes, in the mesh's own
    order and renumbered at random (the detection uses the coordinates, not
    the numbering; the grid variants need the box numbering and exponent 1,
    else they run variant 21), batch 3, Dirichlet values on two faces, loss
    exponents 1 and 1.5: losses and both gradients against the oracle, and
    bit-identical on a repeat call."""
    m = _box_mesh(order)
    s = _settings("hex8", "elastic", "element", exponent)
    gl = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": variant})
    feats = gl.KernelFeatures()
    assert feats["uniform_box"] and feats["box_grid"] == (order == "structured")
    ol = oracle_loss("hex8", "elastic", m, s)
    rng = np.random.default_rng(47)
    ctrl = 0.5 + rng.random((3, gl.GetNumberOfControls()))
    u = 0.01 * rng.standard_normal((3, gl.GetTotalNumberOfDOFs()))
    a = gl.ComputeBatchLossAndGrad(ctrl, u)
    gl.CheckDeviceStatus()
    o = ol.batch_loss_and_grads(ctrl, u)
    for x, z in zip(a[2:], o[2:]):
        assert rel_fro(x.cpu().numpy(), z) < TOL
    assert np.all(a[3].cpu().numpy()[:, ol.dirichlet_indices] == 0)
    b = gl.ComputeBatchLossAndGrad(ctrl, u)
    for x, y in zip(a[2:], b[2:]):
        assert np.array_equal(x.cpu().numpy(), y.cpu().numpy())
    if order == "renumbered":
        assert np.all(a[3].cpu().numpy()[:, -6:] == 0.0)


def test_hex8_box_residual_path_matches_oracle(cuda):
    """The residual-only path (records + node gather, no loss) with a box
    variant chosen."""
    m = _box_mesh()
    s = _settings("hex8", "elastic", "element")
    gl = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": 21})
    ol = oracle_loss("hex8", "elastic", m, s)
    rng = np.random.default_rng(48)
    ctrl = 0.5 + rng.random(gl.GetNumberOfControls())
    uf = ol.full_dof_vector(0.01 * rng.standard_normal(gl.GetTotalNumberOfDOFs()))
    _, R = gl.ComputeJacobianMatrixAndResidualVector(ctrl, uf, with_matrix=False)
    _, Ro = ol.csr(ctrl, uf)
    assert rel_fro(R.cpu().numpy(), Ro) < TOL


@pytest.mark.parametrize("kind", ["jittered", "one_node_moved", "sheared", "nodal", "body_force", "uneven"])
def test_uniform_box_detection_rejects(cuda, kind):
    """The box kernels apply only to identical axis-aligned boxes with
    element controls and no body force; any other mesh or setting keeps the
    pointwise kernels (a box variant then runs variant 16), still exact."""
    m = _box_mesh()
    layout, bf = "element", None
    if kind == "jittered":
        m = make_mesh("hex8", 4, seed=49, jitter=0.1)
    elif kind == "one_node_moved":
        m.nodes_coordinates[20] += np.array([1e-6, 0.0, 0.0])
    elif kind == "sheared":
        m.nodes_coordinates[:, 0] += 0.25 * m.nodes_coordinates[:, 2]
    elif kind == "nodal":
        layout = "nodal"
    elif kind == "body_force":
        bf = [0.1, 0.0, 0.0]
    elif kind == "uneven":
        m = create_3D_box_mesh(4, 4, 4)
        z = m.nodes_coordinates[:, 2]
        m.nodes_coordinates[:, 2] = z * z
    s = _settings("hex8", "elastic", layout, 1.0, bf)
    gl = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": 20})
    assert not gl.KernelFeatures()["uniform_box"]
    ol = oracle_loss("hex8", "elastic", m, s)
    rng = np.random.default_rng(50)
    ctrl = 0.5 + rng.random((2, gl.GetNumberOfControls()))
    u = 0.01 * rng.standard_normal((2, gl.GetTotalNumberOfDOFs()))
    a = gl.ComputeBatchLossAndGrad(ctrl, u)
    o = ol.batch_loss_and_grads(ctrl, u)
    for x, z in zip(a[2:], o[2:]):
        assert rel_fro(x.cpu().numpy(), z) < TOL


@pytest.mark.parametrize("nx,ny,nz", [(37, 19, 11), (16, 8, 4), (17, 9, 5), (1, 1, 7), (40, 2, 3)])
@pytest.mark.parametrize("variant", [23, 24])
def test_hex8_box_grid_tiles_match_oracle(cuda, nx, ny, nz, variant):
    """The one-launch structured grid kernel over many column tiles and layer
    blocks, with uneven last tiles (37 x 19 x 11), a mesh of exactly one tile
    (16 x 8 x 4), one element past it in every direction (17 x 9 x 5), a
    single element column and a thin slab; edge 1/32, batch 2, Dirichlet
    values on the bottom and top faces: losses and both gradients against the
    oracle, bit-identical on a repeat call, and the Dirichlet dofs 0."""
    h = 1.0 / 32
    m = create_3D_box_mesh(nx, ny, nz, Lx=nx * h, Ly=ny * h, Lz=nz * h)
    s = _settings("hex8", "elastic", "element")
    gl = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": variant})
    assert gl.KernelFeatures()["box_grid"]
    ol = oracle_loss("hex8", "elastic", m, s)
    rng = np.random.default_rng(52)
    ctrl = 0.5 + rng.random((2, gl.GetNumberOfControls()))
    u = 0.001 * rng.standard_normal((2, gl.GetTotalNumberOfDOFs()))
    a = gl.ComputeBatchLossAndGrad(ctrl, u)
    gl.CheckDeviceStatus()
    o = ol.batch_loss_and_grads(ctrl, u)
    for x, z in zip(a[2:], o[2:]):
        assert rel_fro(x.cpu().numpy(), z) < TOL
    assert np.all(a[3].cpu().numpy()[:, ol.dirichlet_indices] == 0)
    b = gl.ComputeBatchLossAndGrad(ctrl, u)
    for x, y in zip(a[2:], b[2:]):
        assert np.array_equal(x.cpu().numpy(), y.cpu().numpy())


@pytest.mark.parametrize("variant", [23, 24])
def test_hex8_box_grid_side_face_constraints(cuda, variant):
    """Dirichlet values on the x = 0 and y = 0 faces (a constrained node in
    every node layer, so every layer reads its masks) and on one interior
    node set; the grid kernel against the oracle."""
    h = 1.0 / 16
    m = create_3D_box_mesh(20, 10, 7, Lx=20 * h, Ly=10 * h, Lz=7 * h)
    m.node_sets["mid"] = np.array([37, 555, 901])
    s = _settings("hex8", "elastic", "element")
    s["dirichlet_bc_dict"] = {"Ux": {"left": 0.0, "mid": 0.01}, "Uy": {"front": 0.02}, "Uz": {"left": -0.01}}
    gl = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": variant})
    assert gl.KernelFeatures()["box_grid"]
    ol = oracle_loss("hex8", "elastic", m, s)
    rng = np.random.default_rng(62)
    ctrl = 0.5 + rng.random((2, gl.GetNumberOfControls()))
    u = 0.002 * rng.standard_normal((2, gl.GetTotalNumberOfDOFs()))
    a = gl.ComputeBatchLossAndGrad(ctrl, u)
    gl.CheckDeviceStatus()
    o = ol.batch_loss_and_grads(ctrl, u)
    for x, z in zip(a[2:], o[2:]):
        assert rel_fro(x.cpu().numpy(), z) < TOL
    assert np.all(a[3].cpu().numpy()[:, ol.dirichlet_indices] == 0)


@pytest.mark.parametrize("box", [20, 21, 22, 23, 24])
def test_box_kernel_agrees_with_pointwise_kernel(cuda, box):
    """On a 100^3 cube mesh the box kernels and the pointwise kernel (variant
    11) evaluate the same quadratic form in another order: losses and
    gradients agree to 1e-6."""
    m = create_3D_box_mesh(100, 100, 100)
    s = _settings("hex8", "elastic", "element")
    a_loss = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": box})
    b_loss = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": 11})
    rng = np.random.default_rng(51)
    ctrl = 0.5 + rng.random((2, a_loss.GetNumberOfControls()))
    u = 0.003 * rng.standard_normal((2, a_loss.GetTotalNumberOfDOFs()))
    a = a_loss.ComputeBatchLossAndGrad(ctrl, u)
    b = b_loss.ComputeBatchLossAndGrad(ctrl, u)
    a_loss.CheckDeviceStatus()
    for x, y in zip(a[2:], b[2:]):
        assert rel_fro(x.cpu().numpy(), y.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("tma,twin", [(13, 11), (15, 6), (16, 11), (17, 11)])
@pytest.mark.parametrize("layout", ["nodal", "element"])
def test_tma_variant_equals_its_per_thread_twin(cuda, tma, twin, layout):
    """The persistent TMA-staged kernel runs the same element code as its
    one-element-per-thread twin: on a 100^3 mesh (about 10 tiles per warp, so
    every stage buffer is refilled and its barrier phase flips several times)
    both gradients are bit-identical and the losses (summed in another block
    grouping) agree to 1e-6."""
    m = create_3D_box_mesh(100, 100, 100)
    s = _settings("hex8", "elastic", layout, 1.0, [0.2, 0.0, -0.1])
    a_loss = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": tma})
    b_loss = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": twin})
    rng = np.random.default_rng(29)
    ctrl = 0.5 + rng.random((2, a_loss.GetNumberOfControls()))
    u = 0.003 * rng.standard_normal((2, a_loss.GetTotalNumberOfDOFs()))
    a = a_loss.ComputeBatchLossAndGrad(ctrl, u)
    b = b_loss.ComputeBatchLossAndGrad(ctrl, u)
    a_loss.CheckDeviceStatus()
    assert rel_fro(a[2].cpu().numpy(), b[2].cpu().numpy()) < 1e-6
    assert np.array_equal(a[3].cpu().numpy(), b[3].cpu().numpy())
    assert np.array_equal(a[4].cpu().numpy(), b[4].cpu().numpy())


@pytest.mark.parametrize("layout", ["nodal", "element"])
@pytest.mark.parametrize("B", [1, 3])
def test_pinned_host_buffers_equal_device_buffers(cuda, layout, B):
    """Pinned host inputs (element controls read by the kernel in place) and
    result buffers (the kernels store straight into host memory) give
    bit-identical results to device buffers."""
    torch = cuda
    m = make_mesh("hex8", 6, seed=36, jitter=0.1)
    s = _settings("hex8", "elastic", layout, 1.0)
    gl = gpu_loss("hex8", "elastic", m, s)
    rng = np.random.default_rng(37)
    ctrl = (0.5 + rng.random((B, gl.GetNumberOfControls()))).astype(np.float32)
    u = (0.01 * rng.standard_normal((B, gl.GetTotalNumberOfDOFs()))).astype(np.float32)
    a = gl.ComputeBatchLossAndGrad(torch.from_numpy(ctrl).cuda(), torch.from_numpy(u).cuda())
    out = (torch.empty(B).pin_memory(), torch.empty(B, u.shape[1]).pin_memory(),
           torch.empty(B, ctrl.shape[1]).pin_memory())
    h = gl.ComputeBatchLossAndGrad(torch.from_numpy(ctrl).pin_memory(), torch.from_numpy(u).pin_memory(), out=out)
    torch.cuda.synchronize()  # host results are complete once the stream has finished
    assert np.array_equal(a[0].cpu().numpy(), h[0].cpu().numpy())
    for x, y, o in zip(a[2:], h[2:], out):
        assert y.data_ptr() == o.data_ptr() and not y.is_cuda
        assert np.array_equal(x.cpu().numpy(), y.numpy())
    with pytest.raises(ValueError):
        gl.ComputeBatchLossAndGrad(ctrl, u, out=(torch.empty(B), out[1], out[2]))  # pageable: refused


@pytest.mark.parametrize("B", [1, 3])
def test_host_result_buffers_on_a_grid_plan(cuda, B):
    """A plan on the structured box grid kernel given pinned host inputs and
    result buffers (it then runs the box kernel and the gather, which write
    the gradients over the host link) agrees with the device-buffer call to
    fp32 rounding, and the same tensors passed again (the call reuses its
    validated arguments) give the same results after the inputs change in
    place."""
    torch = cuda
    h = 1.0 / 16
    m = create_3D_box_mesh(20, 12, 9, Lx=20 * h, Ly=12 * h, Lz=9 * h)
    s = _settings("hex8", "elastic", "element", 1.0)
    gl = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": 23})
    assert gl.KernelFeatures()["box_grid"]
    rng = np.random.default_rng(38)
    ctrl = (0.5 + rng.random((B, gl.GetNumberOfControls()))).astype(np.float32)
    u = (0.003 * rng.standard_normal((B, gl.GetTotalNumberOfDOFs()))).astype(np.float32)
    out = (torch.empty(B).pin_memory(), torch.empty(B, u.shape[1]).pin_memory(),
           torch.empty(B, ctrl.shape[1]).pin_memory())
    c_pin, u_pin = torch.from_numpy(ctrl).pin_memory(), torch.from_numpy(u).pin_memory()
    for rep in range(3):
        a = gl.ComputeBatchLossAndGrad(c_pin.cuda(), u_pin.cuda())
        hres = gl.ComputeBatchLossAndGrad(c_pin, u_pin, out=out)
        torch.cuda.synchronize()
        for x, y in zip(a[2:], hres[2:]):
            assert rel_fro(y.cpu().numpy(), x.cpu().numpy()) < 1e-6
        u_pin.mul_(1.5)  # in place: the next call must see the new values
    gl.CheckDeviceStatus()


def test_repeated_call_with_the_same_tensors(cuda):
    """A call with the same tensors as the previous one reuses its validated
    arguments: device inputs changed in place, host inputs changed in place
    (copied again) and a different tensor all give the results of a fresh
    loss object (a stale input would differ by far more than 1e-6); Autotune
    resets the reuse."""
    torch = cuda
    m = make_mesh("hex8", 5, seed=60, jitter=0.05)
    s = _settings("hex8", "elastic", "element")
    gl = gpu_loss("hex8", "elastic", m, s)
    fresh = gpu_loss("hex8", "elastic", m, s)
    rng = np.random.default_rng(61)
    ctrl = torch.tensor(0.5 + rng.random((2, gl.GetNumberOfControls())), dtype=torch.float32, device="cuda")
    u = torch.tensor(0.01 * rng.standard_normal((2, gl.GetTotalNumberOfDOFs())), dtype=torch.float32, device="cuda")
    u_host = u.cpu().pin_memory()
    for step in range(3):
        for args in ((ctrl, u), (ctrl, u_host)):
            a = gl.ComputeBatchLossAndGrad(*args)
            b = fresh.ComputeBatchLossAndGrad(ctrl.clone(), args[1].clone().cuda())
            for x, y in zip(a[2:], b[2:]):  # the autotuned variant rounds differently: 1e-6
                assert rel_fro(x.cpu().numpy(), y.cpu().numpy()) < 1e-6
        u.mul_(1.1)
        u_host.mul_(0.9)
        ctrl.add_(0.05)
        if step == 1:
            gl.Autotune(ctrl, u, repeats=1)
    other = u.clone()
    a = gl.ComputeBatchLossAndGrad(ctrl, other)
    b = fresh.ComputeBatchLossAndGrad(ctrl.clone(), other.clone())
    assert rel_fro(a[3].cpu().numpy(), b[3].cpu().numpy()) < 1e-6


def test_autotune_keeps_results_exact(cuda):
    m = make_mesh("hex8", 6, seed=25)
    s = _settings("hex8", "elastic", "element")
    gl, ol = gpu_loss("hex8", "elastic", m, s), oracle_loss("hex8", "elastic", m, s)
    rng = np.random.default_rng(26)
    ctrl = 0.5 + rng.random((1, gl.GetNumberOfControls()))
    u = 0.01 * rng.standard_normal((1, gl.GetTotalNumberOfDOFs()))
    warm = gl.Autotune(ctrl, u, repeats=2, cold_l2=False)  # back-to-back calls
    nv = HEX8_VARIANTS
    # variants that do not apply to this (jittered) mesh are not timed: -1
    timed = [t for t in warm["ms"] if t >= 0]
    assert 0 <= warm["chosen"] < nv and len(warm["ms"]) == nv and min(timed) > 0 and warm["ms"][warm["chosen"]] > 0
    assert all(t == -1 for t in warm["ms"][20:])
    info = gl.Autotune(ctrl, u, repeats=2)  # every timed call after an L2 flush
    timed = [t for t in info["ms"] if t >= 0]
    assert 0 <= info["chosen"] < nv and len(info["ms"]) == nv and min(timed) > 0 and info["ms"][info["chosen"]] > 0
    a = gl.ComputeBatchLossAndGrad(ctrl, u)
    o = ol.batch_loss_and_grads(ctrl, u)
    for x, z in zip(a[2:], o[2:]):
        assert rel_fro(x.cpu().numpy(), z) < TOL


def test_autotune_keeps_a_forced_variant(cuda):
    m = make_mesh("hex8", 4, seed=27)
    s = _settings("hex8", "elastic", "element")
    gl = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": 3})
    rng = np.random.default_rng(28)
    ctrl = 0.5 + rng.random((1, gl.GetNumberOfControls()))
    u = 0.01 * rng.standard_normal((1, gl.GetTotalNumberOfDOFs()))
    info = gl.Autotune(ctrl, u, repeats=2)
    assert info["chosen"] == 3 and len(info["ms"]) == 1 and info["ms"][0] > 0


@pytest.mark.parametrize("exponent,bf", [(1.5, None), (1.0, [0.3, -0.2, 0.1]), (2.0, [0.1, 0.2, 0.3])])
def test_loss_exponent_body_force_broadcast(cuda, exponent, bf):
    m = make_mesh("hex8", 3, seed=3)
    s = _settings("hex8", "elastic", "nodal", exponent, bf)
    gl, ol = gpu_loss("hex8", "elastic", m, s), oracle_loss("hex8", "elastic", m, s)
    rng = np.random.default_rng(4)
    ctrl = 0.5 + rng.random((1, m.GetNumberOfNodes()))          # one control broadcast to every instance
    u = 0.05 * rng.standard_normal((3, gl.GetTotalNumberOfDOFs()))
    _, _, losses, du, dc = gl.ComputeBatchLossAndGrad(ctrl, u)
    _, _, olosses, odu, odc = ol.batch_loss_and_grads(np.repeat(ctrl, 3, 0), u)
    assert rel_fro(losses.cpu().numpy(), olosses) < TOL
    assert rel_fro(du.cpu().numpy(), odu) < TOL
    assert rel_fro(dc.cpu().numpy(), odc) < TOL


@pytest.mark.parametrize("etype,physics", [("hex8", "elastic"), ("quad4", "thermal"), ("tet4", "elastic")])
@pytest.mark.parametrize("layout", ["nodal", "element"])
def test_plain_path_matches_fused(cuda, etype, physics, layout):
    m = make_mesh(etype, 4 if etype != "quad4" else 10, seed=5)
    s = _settings(etype, physics, layout, 1.0, [0.1, 0.0, -0.2] if physics == "elastic" else None)
    gl = gpu_loss(etype, physics, m, s)
    rng = np.random.default_rng(6)
    ctrl = 0.5 + rng.random((2, gl.GetNumberOfControls()))
    u = 0.05 * rng.standard_normal((2, gl.GetTotalNumberOfDOFs()))
    f = gl.ComputeBatchLossAndGrad(ctrl, u)
    p = gl.ComputeBatchLossAndGrad(ctrl, u, plain=True)
    for a, b in zip(f[2:], p[2:]):
        assert rel_fro(a.cpu().numpy(), b.cpu().numpy()) < TOL


def test_fused_is_deterministic(cuda):
    m = make_mesh("hex8", 6, seed=7)
    gl = gpu_loss("hex8", "elastic", m, _settings("hex8", "elastic"))
    rng = np.random.default_rng(8)
    ctrl = 0.5 + rng.random((1, m.GetNumberOfNodes()))
    u = 0.05 * rng.standard_normal((1, gl.GetTotalNumberOfDOFs()))
    a = [t.clone() for t in gl.ComputeBatchLossAndGrad(ctrl, u)[2:]]
    b = gl.ComputeBatchLossAndGrad(ctrl, u)[2:]
    for x, y in zip(a, b):
        assert cuda.equal(x, y)


@pytest.mark.parametrize("etype,physics,n", [("quad4", "thermal", 6), ("hex8", "elastic", 3), ("tet4", "neohooke", 2),
                                             ("quad4", "elastic", 5), ("hex8", "neohooke", 2), ("tet4", "thermal", 2)])
@pytest.mark.parametrize("transpose", [False, True])
def test_csr_pattern_bit_exact_and_values(cuda, etype, physics, n, transpose):
    """Pattern identical to scipy.sparse.csr_array of the reference COO
    (fe_solver.py:71-72); values and residual within 1e-5."""
    m = make_mesh(etype, n, seed=9)
    s = _settings(etype, physics, "nodal", 1.0, [0.2, 0.1, 0.0] if physics != "thermal" else None)
    gl, ol = gpu_loss(etype, physics, m, s), oracle_loss(etype, physics, m, s)
    rng = np.random.default_rng(10)
    ctrl = 0.5 + rng.random(m.GetNumberOfNodes())
    u = ol.full_dof_vector((0.03 / n) * rng.standard_normal(ol.total_dofs))
    jac, R = gl.ComputeJacobianMatrixAndResidualVector(ctrl, u, transpose_jacobian=transpose)
    gl.CheckDeviceStatus()
    A, Ro = ol.csr(ctrl, u, transpose=transpose)
    np.testing.assert_array_equal(jac.indptr.cpu().numpy(), A.indptr)
    np.testing.assert_array_equal(jac.indices.cpu().numpy(), A.indices)
    assert rel_fro(jac.data.cpu().numpy(), A.data) < TOL
    assert rel_fro(R.cpu().numpy(), Ro) < TOL
    np.testing.assert_allclose(jac.inv_diag.cpu().numpy(), 1.0 / A.diagonal(), rtol=1e-5)


def test_spmv_matches_scipy(cuda):
    m = make_mesh("hex8", 5, seed=11)
    s = _settings("hex8", "elastic")
    gl, ol = gpu_loss("hex8", "elastic", m, s), oracle_loss("hex8", "elastic", m, s)
    ctrl = 0.5 + np.random.default_rng(12).random(m.GetNumberOfNodes())
    jac, _ = gl.ComputeJacobianMatrixAndResidualVector(ctrl, np.zeros(ol.total_dofs))
    x = np.random.default_rng(13).standard_normal(ol.total_dofs)
    y = jac.matvec(x).cpu().numpy()
    assert rel_fro(y, jac.to_scipy() @ x) < TOL


@pytest.mark.parametrize("etype,physics,n", [("hex8", "elastic", 8), ("quad4", "thermal", 40), ("tet4", "elastic", 5)])
def test_linear_solve_matches_direct(cuda, etype, physics, n):
    """FiniteElementLinearResidualBasedSolver.Solve (PCG, rtol 1e-8) against an
    FP64 direct solve of the oracle system: within 1e-6 relative."""
    from folax_gb300.solvers import FiniteElementLinearResidualBasedSolver
    m = make_mesh(etype, n, seed=14)
    s = _settings(etype, physics)
    gl, ol = gpu_loss(etype, physics, m, s), oracle_loss(etype, physics, m, s)
    ctrl = 0.5 + np.random.default_rng(15).random(m.GetNumberOfNodes())
    solver = FiniteElementLinearResidualBasedSolver("lin", gl, {"linear_solver_settings": {"solver": "GB300-pcg", "tol": 1e-8, "maxiter": 5000}})
    solver.Initialize()
    x = solver.Solve(ctrl, np.zeros(ol.total_dofs)).cpu().numpy()
    xo = fo.linear_solve(ol, ctrl, np.zeros(ol.total_dofs))
    info = solver.last_linear_info
    assert info["status"] == 0, info
    assert rel_fro(x, xo) < 1e-6, (rel_fro(x, xo), info)


def test_newton_neohooke_matches_oracle(cuda):
    from folax_gb300.solvers import FiniteElementNonLinearResidualBasedSolver
    m = make_mesh("tet4", 3, seed=16)
    s = _settings("tet4", "neohooke", shear="consistent")
    gl, ol = gpu_loss("tet4", "neohooke", m, s), oracle_loss("tet4", "neohooke", m, s)
    ctrl = 0.5 + np.random.default_rng(17).random(m.GetNumberOfNodes())
    settings = {"linear_solver_settings": {"tol": 1e-10, "maxiter": 5000},
                "nonlinear_solver_settings": {"load_incr": 2, "maxiter": 10, "abs_tol": 1e-6, "rel_tol": 1e-7}}
    solver = FiniteElementNonLinearResidualBasedSolver("nl", gl, settings)
    solver.Initialize()
    x = solver.Solve(ctrl, np.zeros(ol.total_dofs)).cpu().numpy()
    xo, _ = fo.newton_solve(ol, ctrl, np.zeros(ol.total_dofs), load_incr=2, maxiter=10, abs_tol=1e-6, rel_tol=1e-7)
    assert rel_fro(x, xo) < 1e-5
    # the Newton root of the consistent residual minimises the loss: its gradient vanishes
    _, _, _, du, _ = gl.ComputeBatchLossAndGrad(ctrl[None], x[None])
    _, _, _, du0, _ = gl.ComputeBatchLossAndGrad(ctrl[None], np.zeros((1, ol.total_dofs)))
    assert cuda.linalg.vector_norm(du) < 1e-3 * cuda.linalg.vector_norm(du0)


def test_bounded_wait_gives_up_and_reports(cuda):
    """A TMA-stage wait whose copy never comes (an mbarrier with announced
    bytes and no copy) gives up after its poll limit: the status word gets
    FOLGB_ERR_TIMEOUT and the context stays usable."""
    import time
    from folax_gb300 import _capi
    torch = cuda
    lib = _capi.load()
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    t0 = time.perf_counter()
    assert lib.folgb_selftest_bounded_wait(_capi.ptr(status), _capi.stream_handle()) == 0
    torch.cuda.synchronize()
    assert time.perf_counter() - t0 < 30.0
    assert int(status.item()) == 1 << _capi.ERR_TIMEOUT
    m = make_mesh("hex8", 3, seed=66)
    gl = gpu_loss("hex8", "elastic", m, _settings("hex8", "elastic"))
    _, _, losses, _, _ = gl.ComputeBatchLossAndGrad(np.ones((1, gl.GetNumberOfControls())),
                                                    np.zeros((1, gl.GetTotalNumberOfDOFs())))
    assert np.isfinite(losses.cpu().numpy()).all()


def test_inverted_element_and_nan_are_reported(cuda):
    """Host-made faults: an inverted element raises the detJ status bit, a NaN
    in u the NaN bit; the context stays usable."""
    from folax_gb300 import _capi
    m = make_mesh("hex8", 2, seed=18, jitter=0.0)
    conn = m.elements_nodes["hexahedron"].copy()
    conn[0, [0, 1]] = conn[0, [1, 0]]
    m.elements_nodes["hexahedron"] = conn
    gl = gpu_loss("hex8", "elastic", m, _settings("hex8", "elastic"))
    u = np.zeros((1, gl.GetTotalNumberOfDOFs()))
    ctrl = np.ones((1, m.GetNumberOfNodes()))
    gl.ComputeBatchLossAndGrad(ctrl, u)
    with pytest.raises(_capi.FolgbError) as e:
        gl.CheckDeviceStatus()
    assert e.value.code == _capi.ERR_NONPOSITIVE_DETJ
    m2 = make_mesh("hex8", 2, seed=18)
    gl2 = gpu_loss("hex8", "elastic", m2, _settings("hex8", "elastic"))
    free = gl2.non_dirichlet_indices[len(gl2.non_dirichlet_indices) // 2]
    u[0, free] = np.nan
    gl2.ComputeBatchLossAndGrad(ctrl, u)
    with pytest.raises(_capi.FolgbError) as e:
        gl2.CheckDeviceStatus()
    assert e.value.code == _capi.ERR_NAN
    gl2.ComputeBatchLossAndGrad(ctrl, np.zeros_like(u))
    gl2.CheckDeviceStatus()


def test_invalid_arguments_raise(cuda):
    from folax_gb300 import _capi
    m = make_mesh("quad4", 3)
    m.elements_nodes["quad"] = m.elements_nodes["quad"].copy()
    m.elements_nodes["quad"][0, 0] = 10 ** 6          # node id out of range
    with pytest.raises(_capi.FolgbError):
        gpu_loss("quad4", "thermal", m, _settings("quad4", "thermal"))


@pytest.mark.parametrize("shear", ["reference", "consistent"])
def test_bicgstab_on_indefinite_neohooke_tangent(cuda, shear):
    """The reference NH model is not stress-free at C = I (S = -mu I), so its
    tangent is indefinite near u = 0: Jacobi-BiCGSTAB (the reference's default
    solver) against an FP64 direct solve."""
    from folax_gb300.solvers import FiniteElementSolver
    m = make_mesh("tet4", 3, seed=19)
    s = _settings("tet4", "neohooke", shear=shear)
    gl, ol = gpu_loss("tet4", "neohooke", m, s), oracle_loss("tet4", "neohooke", m, s)
    ctrl = 0.5 + np.random.default_rng(20).random(m.GetNumberOfNodes())
    u = ol.full_dof_vector(np.zeros(ol.total_dofs), 0.5)
    jac, R = gl.ComputeJacobianMatrixAndResidualVector(ctrl, u)
    solver = FiniteElementSolver("b", gl, {"linear_solver_settings": {"solver": "JAX-bicgstab", "tol": 1e-9,
                                                                       "maxiter": 4000}})
    solver.Initialize()
    dx = solver.LinearSolve(jac, R).cpu().numpy()
    A, Ro = ol.csr(ctrl, u)
    assert solver.last_linear_info["status"] == 0, solver.last_linear_info
    assert rel_fro(dx, fo.direct_solve(A, -Ro)) < 1e-5


@pytest.mark.parametrize("bits", [32, 64])
def test_krylov_vector_precision_on_spd_system(cuda, bits):
    """folgb_krylov: CG with fp32 or fp64 Krylov vectors on an SPD stiffness."""
    from folax_gb300.solvers import FiniteElementSolver
    m = make_mesh("hex8", 6, seed=51)
    s = _settings("hex8", "elastic", "element")
    gl, ol = gpu_loss("hex8", "elastic", m, s), oracle_loss("hex8", "elastic", m, s)
    ctrl = 0.5 + np.random.default_rng(52).random(gl.GetNumberOfControls())
    u = ol.full_dof_vector(np.zeros(ol.total_dofs))
    jac, R = gl.ComputeJacobianMatrixAndResidualVector(ctrl, u)
    solver = FiniteElementSolver("cg", gl, {"linear_solver_settings": {
        "solver": "GB300-pcg", "tol": 1e-8, "maxiter": 5000, "vector_precision": f"fp{bits}"}})
    solver.Initialize()
    dx = solver.LinearSolve(jac, R).cpu().numpy()
    assert solver.last_linear_info["status"] == 0 and solver.last_linear_info["vector_bits"] == bits
    A, Ro = ol.csr(ctrl, u)
    assert rel_fro(dx, fo.direct_solve(A, -Ro)) < 1e-5


def test_fp64_vector_bicgstab_on_12cubed_neohooke_tangent(cuda):
    """The first Newton tangent of the Neo-Hookean tet split of a 12^3 grid
    (two-phase E, reference shear): fp32 BiCGSTAB recurrences diverge on it;
    with fp64 vectors the solve converges (rtol 1e-6 on the fp64 iterate) and
    the returned fp32 solution's residual against the GPU's own matrix is at
    the fp32 rounding floor of the exact solution."""
    from folax_gb300 import fields
    from folax_gb300.mesh import create_3D_box_mesh, split_hex_to_tets
    from folax_gb300.solvers import FiniteElementSolver
    n = 12
    m = split_hex_to_tets(create_3D_box_mesh(n, n, n))
    s = {"dirichlet_bc_dict": {"Ux": {"bottom": 0.0}, "Uy": {"bottom": 0.0}, "Uz": {"bottom": 0.0, "top": 0.05}},
         "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3}, "control_layout": "element"}
    gl = gpu_loss("tet4", "neohooke", m, s)
    E = np.repeat(fields.two_phase_voxels(n, 2024), 6)
    u = gl.ApplyDirichletBCOnDofVector(np.zeros(gl.GetTotalNumberOfDOFs()))
    jac, R = gl.ComputeJacobianMatrixAndResidualVector(E, u)
    solver = FiniteElementSolver("b", gl, {"linear_solver_settings": {"solver": "JAX-bicgstab", "tol": 1e-6,
                                                                       "maxiter": 20000, "check_every": 64}})
    solver.Initialize()
    dx = solver.LinearSolve(jac, R).double().cpu().numpy()
    info = solver.last_linear_info
    assert info["vector_bits"] == 64 and info["status"] == 0, info
    A = jac.to_scipy()
    r = R.double().cpu().numpy()
    # the solution comes back in fp32: its rounding alone leaves a residual
    # floor on this ill-conditioned system, measured on the exact solution
    x_star = fo.direct_solve(A, -r)
    floor = np.linalg.norm(A @ x_star.astype(np.float32).astype(np.float64) + r) / np.linalg.norm(r)
    res = np.linalg.norm(A @ dx + r) / np.linalg.norm(r)
    assert res < 1e-6 + 2.0 * floor, (res, floor)


def test_newton_neohooke_reference_shear_two_phase_matches_oracle(cuda):
    """Newton (load_incr 1) on the reference Neo-Hookean model, 6^3 tet split,
    two-phase E: the GPU path (fp32 assembly, fp64-vector BiCGSTAB) converges
    to the oracle's root (FP64 assembly, direct solves)."""
    from folax_gb300 import fields
    from folax_gb300.mesh import create_3D_box_mesh, split_hex_to_tets
    from folax_gb300.solvers import FiniteElementNonLinearResidualBasedSolver
    n = 6
    m = split_hex_to_tets(create_3D_box_mesh(n, n, n))
    s = {"dirichlet_bc_dict": {"Ux": {"bottom": 0.0}, "Uy": {"bottom": 0.0}, "Uz": {"bottom": 0.0, "top": 0.05}},
         "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3}, "control_layout": "element"}
    gl, ol = gpu_loss("tet4", "neohooke", m, s), oracle_loss("tet4", "neohooke", m, s)
    E = np.repeat(fields.two_phase_voxels(n, 2024), 6)
    solver = FiniteElementNonLinearResidualBasedSolver("nl", gl, {
        "linear_solver_settings": {"tol": 1e-9, "maxiter": 20000, "check_every": 64},
        "nonlinear_solver_settings": {"load_incr": 1, "maxiter": 12, "abs_tol": 1e-7, "rel_tol": 1e-8}})
    solver.Initialize()
    x = solver.Solve(E, np.zeros(ol.total_dofs)).double().cpu().numpy()
    xo, _ = fo.newton_solve(ol, E, np.zeros(ol.total_dofs), load_incr=1, maxiter=12, abs_tol=1e-7, rel_tol=1e-8)
    assert rel_fro(x, xo) < 1e-4


@pytest.mark.parametrize("solver_name", ["GB300-pcg", "JAX-bicgstab"])
def test_device_resident_krylov_loop_matches_host_loop(cuda, solver_name):
    """The solve loop as one CUDA graph (WHILE node, no host sync until the
    end) runs the same kernels in the same order as the host-driven loop
    (forced here by enabling kernel tracing): bit-identical results.  32^3
    hex8 (107,811 dofs) is above the size the single-cluster solver takes;
    the kernel-loop engine is selected, since the grid engine (one launch)
    sums its reductions in another order."""
    from folax_gb300 import _capi
    from folax_gb300.solvers import FiniteElementSolver
    torch = cuda
    m = make_mesh("hex8", 32, seed=61)
    s = _settings("hex8", "elastic", "element")
    gl = gpu_loss("hex8", "elastic", m, s)
    ctrl = 0.5 + np.random.default_rng(62).random(gl.GetNumberOfControls())
    u = gl.ApplyDirichletBCOnDofVector(np.zeros(gl.GetTotalNumberOfDOFs()))
    jac, R = gl.ComputeJacobianMatrixAndResidualVector(ctrl, u)
    solver = FiniteElementSolver("k", gl, {"linear_solver_settings": {"solver": solver_name, "tol": 1e-8,
                                                                       "maxiter": 5000, "check_every": 32}})
    solver.Initialize()
    lib = _capi.load()
    lib.folgb_krylov_set_engine(_capi.KRYLOV_ENGINE_KERNELS)
    try:
        x_dev = solver.LinearSolve(jac, R)
        info_dev = dict(solver.last_linear_info)
        lib.folgb_trace_enable(1)
        x_host = solver.LinearSolve(jac, R)
    finally:
        lib.folgb_trace_enable(0)
        lib.folgb_krylov_set_engine(_capi.KRYLOV_ENGINE_GRID)
    info_host = dict(solver.last_linear_info)
    assert info_dev["status"] == 0 and info_dev["iterations"] == info_host["iterations"]
    assert torch.equal(x_dev, x_host)


@pytest.mark.parametrize("etype,physics,n,solver_name,bits", [("hex8", "saint_venant", 14, "JAX-bicgstab", "fp32"),
                                                               ("tet4", "neohooke_split", 4, "JAX-bicgstab", "fp64"),
                                                               ("quad4", "neohooke", 8, "JAX-bicgstab", "fp64"),
                                                               ("hex8", "elastic", 14, "GB300-pcg", "fp32")])
def test_device_resident_newton_matches_host_loop(cuda, etype, physics, n, solver_name, bits):
    """The whole Newton solve as one CUDA graph (WHILE over Newton iterations,
    a nested WHILE over Krylov iterations, no host synchronisation until it
    ends) against the host-driven Newton loop: the same iteration sequence
    and residual history, and the same root within the Krylov tolerance.  14^3
    hex8 (10,125 dofs) runs the host loop's linear solves in the
    single-cluster solver, so the Krylov arithmetic differs; 4^3 tets and the
    fp64-vector solves share it."""
    from folax_gb300.solvers import FiniteElementNonLinearResidualBasedSolver
    m = make_mesh(etype, n, seed=63)
    s = _settings(etype, physics, "nodal")
    gl = gpu_loss(etype, physics, m, s)
    ctrl = 0.5 + np.random.default_rng(64).random(gl.GetNumberOfControls())
    out = {}
    for resident in (True, False):
        solver = FiniteElementNonLinearResidualBasedSolver("nl", gl, {
            "linear_solver_settings": {"solver": solver_name, "tol": 1e-10, "maxiter": 5000, "vector_precision": bits},
            "nonlinear_solver_settings": {"load_incr": 2, "maxiter": 8, "abs_tol": 1e-7, "rel_tol": 1e-8,
                                          "device_resident": resident}})
        solver.Initialize()
        x = solver.Solve(ctrl, np.zeros(gl.GetTotalNumberOfDOFs())).double().cpu().numpy()
        out[resident] = (x, [(h["load_step"], h["iteration"], h["res_norm"]) for h in solver.history])
    (xd, hd), (xh, hh) = out[True], out[False]
    assert [h[:2] for h in hd] == [h[:2] for h in hh]
    np.testing.assert_allclose([h[2] for h in hd], [h[2] for h in hh], rtol=1e-3, atol=1e-9)
    assert rel_fro(xd, xh) < 1e-6


def test_device_resident_newton_reports_nan(cuda):
    """A NaN in the control makes |r| non-finite: the device-resident solve
    stops and raises like the reference's host check."""
    from folax_gb300.solvers import FiniteElementNonLinearResidualBasedSolver
    m = make_mesh("hex8", 3, seed=65)
    s = _settings("hex8", "elastic", "nodal")
    gl = gpu_loss("hex8", "elastic", m, s)
    ctrl = np.ones(gl.GetNumberOfControls())
    ctrl[5] = np.nan
    solver = FiniteElementNonLinearResidualBasedSolver("nl", gl, {"nonlinear_solver_settings": {"load_incr": 2}})
    solver.Initialize()
    with pytest.raises(ValueError):
        solver.Solve(ctrl, np.zeros(gl.GetTotalNumberOfDOFs()))
    assert solver.last_newton_info["newton_iterations"] == 1
    gl._status.zero_()  # the assembly also raised the NaN status bit
    # the context is still usable
    x = FiniteElementNonLinearResidualBasedSolver("nl2", gl, {"nonlinear_solver_settings": {"load_incr": 1}})
    x.Initialize()
    assert np.isfinite(x.Solve(np.ones(gl.GetNumberOfControls()), np.zeros(gl.GetTotalNumberOfDOFs())).cpu().numpy()).all()


@pytest.mark.parametrize("solver_name,etype,physics,n", [("GB300-pcg", "hex8", "elastic", 8),
                                                        ("GB300-pcg", "quad4", "thermal", 50),
                                                        ("JAX-bicgstab", "tet4", "elastic", 6),
                                                        ("JAX-bicgstab", "quad4", "elastic", 24)])
def test_cluster_solver_matches_direct_solve(cuda, solver_name, etype, physics, n):
    """Systems up to 16,384 dofs with fp32 Krylov vectors are solved in one
    thread-block-cluster launch (all phases separated by cluster barriers,
    reductions over distributed shared memory): against an FP64 direct solve,
    and deterministic."""
    from folax_gb300.solvers import FiniteElementSolver
    torch = cuda
    m = make_mesh(etype, n, seed=63)
    s = _settings(etype, physics, "nodal")
    gl, ol = gpu_loss(etype, physics, m, s), oracle_loss(etype, physics, m, s)
    ctrl = 0.5 + np.random.default_rng(64).random(gl.GetNumberOfControls())
    u = ol.full_dof_vector(np.zeros(ol.total_dofs))
    jac, R = gl.ComputeJacobianMatrixAndResidualVector(ctrl, u)
    solver = FiniteElementSolver("k", gl, {"linear_solver_settings": {"solver": solver_name, "tol": 1e-8,
                                                                       "maxiter": 20000, "vector_precision": "fp32"}})
    solver.Initialize()
    x1 = solver.LinearSolve(jac, R)
    assert solver.last_linear_info["status"] == 0, solver.last_linear_info
    x2 = solver.LinearSolve(jac, R)
    assert torch.equal(x1, x2)
    A, Ro = ol.csr(ctrl, u)
    assert rel_fro(x1.cpu().numpy(), fo.direct_solve(A, -Ro)) < 1e-5


@pytest.mark.parametrize("etype,n", [("quad4", 6), ("tet4", 2), ("hex8", 3)])
@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("physics", ["thermal", "elastic"])
def test_every_gauss_order_matches_oracle(cuda, etype, n, order, physics):
    """Gauss orders 1-3 (fe_loss.py:68-83): the compile-time rules (quad4 2x2,
    tet4 1-point) and the run-time tables give the oracle's loss, gradients,
    residual and tangent, batched and single."""
    m = make_mesh(etype, n, seed=40 + order)
    s = {**_settings(etype, physics, "nodal"), "num_gp": order}
    gl, ol = gpu_loss(etype, physics, m, s), oracle_loss(etype, physics, m, s)
    rng = np.random.default_rng(50 + order)
    ctrl = 0.5 + rng.random((2, gl.GetNumberOfControls()))
    u = (0.05 / n) * rng.standard_normal((2, gl.GetTotalNumberOfDOFs()))
    a = gl.ComputeBatchLossAndGrad(ctrl, u)
    o = ol.batch_loss_and_grads(ctrl, u)
    gl.CheckDeviceStatus()
    for x, z in zip(a[2:], o[2:]):
        assert rel_fro(x.cpu().numpy(), z) < TOL
    uf = ol.full_dof_vector(u[0])
    jac, R = gl.ComputeJacobianMatrixAndResidualVector(ctrl[0], uf)
    A, Ro = ol.csr(ctrl[0], uf)
    assert rel_fro(jac.data.cpu().numpy(), A.data) < TOL
    assert rel_fro(R.cpu().numpy(), Ro) < TOL
