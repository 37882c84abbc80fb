"""Host-side logic (CPU): mesh orderings, node sets, tet split, fields,
Dirichlet bookkeeping, settings merging."""
import numpy as np

from folax_gb300 import fields
from folax_gb300 import mesh as M
from folax_gb300.solvers import UpdateDefaultDict
from oracle import fe_oracle as fo


def test_square_mesh_matches_reference_ordering():
    m = M.create_2D_square_mesh(1.0, 6)
    xyz, conn, sets = fo.square_mesh(1.0, 6)
    np.testing.assert_array_equal(m.elements_nodes["quad"], conn)
    np.testing.assert_allclose(m.nodes_coordinates, xyz)
    np.testing.assert_array_equal(m.node_sets["left"], sets["left"])
    np.testing.assert_array_equal(m.node_sets["right"], sets["right"])


def test_box_mesh_positive_jacobians_and_sets():
    m = M.create_3D_box_mesh(3, 4, 5, 1.0, 2.0, 3.0)
    conn = m.elements_nodes["hexahedron"]
    assert conn.shape == (60, 8)
    assert np.all(M.element_jacobian_det("hexahedron", m.nodes_coordinates, conn) > 0)
    assert np.allclose(m.nodes_coordinates[m.node_sets["top"], 2], 3.0)
    assert np.allclose(m.nodes_coordinates[m.node_sets["right"], 0], 1.0)
    assert len(m.node_sets["bottom"]) == 4 * 5


def test_tet_split_conforming_and_oriented():
    m = M.split_hex_to_tets(M.create_3D_box_mesh(3, 3, 3))
    tets = m.elements_nodes["tetra"]
    assert tets.shape == (6 * 27, 4)
    assert np.all(M.element_jacobian_det("tetra", m.nodes_coordinates, tets) > 0)
    # total volume = 1 and every interior face is shared by exactly two tets
    X = m.nodes_coordinates[tets]
    vol = np.abs(np.linalg.det(np.stack([X[:, 1] - X[:, 0], X[:, 2] - X[:, 0], X[:, 3] - X[:, 0]], 2))) / 6
    np.testing.assert_allclose(vol.sum(), 1.0)
    faces = np.sort(np.concatenate([tets[:, [0, 1, 2]], tets[:, [0, 1, 3]], tets[:, [0, 2, 3]], tets[:, [1, 2, 3]]]), 1)
    _, counts = np.unique(faces, axis=0, return_counts=True)
    assert set(counts.tolist()) <= {1, 2}


def test_orientation_fix():
    m = M.create_3D_box_mesh(1, 1, 1)
    conn = m.elements_nodes["hexahedron"].copy()
    conn[0, [0, 1]] = conn[0, [1, 0]]
    m.elements_nodes["hexahedron"] = conn
    m.is_initialized = False
    m.Initialize()
    assert M.element_jacobian_det("hexahedron", m.nodes_coordinates, m.elements_nodes["hexahedron"])[0] > 0


def test_fields_deterministic_and_bounded():
    m = M.create_2D_square_mesh(1.0, 11)
    c = fields.element_centroids(m.nodes_coordinates, m.elements_nodes["quad"])
    k1 = fields.fourier_conductivity(c, seed=3)
    k2 = fields.fourier_conductivity(c, seed=3)
    np.testing.assert_array_equal(k1, k2)
    assert k1.min() >= 0.1 and k1.max() <= 1.0
    v = fields.two_phase_voxels(32, seed=5)
    assert set(np.unique(v)) <= {0.1, 1.0}
    assert 0.1 < (v == 1.0).mean() < 0.9


def test_update_default_dict_drops_unknown_keys():
    d = UpdateDefaultDict({"a": 1, "b": 2}, {"b": 3, "c": 4})
    assert d == {"a": 1, "b": 3}


def test_oracle_fourier_control_matches_formula():
    m = M.create_2D_square_mesh(1.0, 4)
    freqs = fo.fourier_frequencies([2, 4], [2], [0])
    v = np.array([0.3, 0.5, -0.2])
    X = np.zeros((m.GetNumberOfNodes(), 3))
    X[:, :2] = m.nodes_coordinates[:, :2]
    K = 0.15 + 0.5 * np.cos(2 * np.pi * X[:, 0]) * np.cos(2 * np.pi * X[:, 1]) \
        - 0.2 * np.cos(4 * np.pi * X[:, 0]) * np.cos(2 * np.pi * X[:, 1])
    got = fo.fourier_control_values(v, freqs, X, vmin=0.1, vmax=1.0, beta=20)
    np.testing.assert_allclose(got[0], 0.9 / (1 + np.exp(-20 * (K - 0.5))) + 0.1)


def test_oracle_fourier_control_vjp_matches_central_differences():
    rng = np.random.default_rng(8)
    X = rng.random((40, 3))
    freqs = fo.fourier_frequencies([1, 2], [0, 3], [1])
    c = 0.3 * rng.standard_normal((2, len(freqs) + 1))
    dv = rng.standard_normal((2, 40))
    kw = dict(vmin=0.1, vmax=2.0, beta=3.0, scale_min=-0.5, scale_max=1.5)
    g = fo.fourier_control_vjp(c, dv, freqs, X, **kw)
    h = 1e-6
    for b in range(2):
        for q in range(c.shape[1]):
            cp, cm = c.copy(), c.copy()
            cp[b, q] += h
            cm[b, q] -= h
            fd = (np.sum(dv[b] * fo.fourier_control_values(cp[b], freqs, X, **kw)[0])
                  - np.sum(dv[b] * fo.fourier_control_values(cm[b], freqs, X, **kw)[0])) / (2 * h)
            assert abs(fd - g[b, q]) < 1e-7 * max(1.0, abs(fd))


def test_python_mirrors_of_library_constants():
    """The host's variant count, variant names and batched tile sizes are the
    ones the CUDA sources define (kHex8Variants, kBatchTiles)."""
    import os
    import re
    from conftest import ROOT
    from folax_gb300.batched import BatchedFELoss
    from folax_gb300.loss import HEX8_VARIANT_NAMES, HEX8_VARIANTS
    csrc = os.path.join(ROOT, "folax_gb300", "csrc")
    hex8 = open(os.path.join(csrc, "hex8_fused.cu")).read()
    assert int(re.search(r"constexpr int kHex8Variants = (\d+);", hex8).group(1)) == HEX8_VARIANTS
    assert len(HEX8_VARIANT_NAMES) == HEX8_VARIANTS
    batched = open(os.path.join(csrc, "batched.cu")).read()
    tiles = re.search(r"constexpr int kBatchTiles\[\] = \{([^}]*)\};", batched).group(1)
    assert tuple(int(t) for t in tiles.split(",")) == BatchedFELoss.BATCH_TILES
