"""Kratos .mdpa mesh reading (fol/mesh_input_output/mesh.py:93-110, 196-242):
the reference's own fixture with the counts its test asserts
(tests/unit/test_mesh_io.py:26-29), a round trip through a file this test
writes (several element blocks, nested SubModelParts, non-consecutive node
ids, elements that need re-orientation), and the FE loss on the reference's
unstructured tetrahedral mesh on the GPU against the FP64 oracle."""
import numpy as np
import pytest

from conftest import GOLDEN, golden
from folax_gb300.mesh import Mesh, create_3D_box_mesh, element_jacobian_det, split_hex_to_tets


def _sphere():
    g = golden("mesh_io.json")
    m = Mesh("mdpa_io", file_name=g["file"], case_dir=GOLDEN)
    m.Initialize()
    return g, m


def test_reference_fixture_counts():
    g, m = _sphere()
    assert m.GetNumberOfNodes() == g["num_nodes"]["value"]
    assert m.GetNumberOfElements(g["num_elements"]["type"]) == g["num_elements"]["value"]
    for name, entry in g["node_sets"].items():
        assert len(m.GetNodeSet(name)) == entry["value"]
    conn = m.GetElementsNodes("tetra")
    assert conn.min() >= 0 and conn.max() < m.GetNumberOfNodes()
    assert (element_jacobian_det("tetra", m.GetNodesCoordinates(), conn) > 0).all()


def _write_mdpa(path, xyz, ids, blocks, parts):
    with open(path, "w") as f:
        f.write("Begin ModelPartData\n//  VARIABLE_NAME value\nEnd ModelPartData\n\n")
        f.write("Begin Properties 0\nEnd Properties\n\nBegin Nodes\n")
        for i, (x, y, z) in zip(ids, xyz):
            f.write(f"   {i}  {x:.17g}  {y:.17g}  {z:.17g}\n")
        f.write("End Nodes\n\n")
        eid = 1
        for name, conn in blocks:
            f.write(f"Begin Elements {name}// GUI group identifier: block\n")
            for row in conn:
                f.write(f"  {eid} 0 " + " ".join(str(ids[n]) for n in row) + "\n")
                eid += 1
            f.write("End Elements\n\n")
        for name, nodes, nested in parts:
            f.write(f"Begin SubModelPart {name}\n    Begin SubModelPartNodes\n")
            for n in nodes:
                f.write(f"        {ids[n]}\n")
            f.write("    End SubModelPartNodes\n    Begin SubModelPartElements\n    End SubModelPartElements\n")
            if nested:
                f.write("    Begin SubModelPart inner\n        Begin SubModelPartNodes\n            "
                        f"{ids[nodes[0]]}\n        End SubModelPartNodes\n    End SubModelPart\n")
            f.write("    Begin SubModelPartConditions\n    End SubModelPartConditions\nEnd SubModelPart\n\n")


def test_round_trip_with_orientation_and_scale(tmp_path):
    box = create_3D_box_mesh(3, 2, 2)
    tets = split_hex_to_tets(box)
    xyz = box.nodes_coordinates
    ids = 10 + 3 * np.arange(len(xyz))  # non-consecutive Kratos ids
    tconn = tets.elements_nodes["tetra"].copy()
    flipped = tconn.copy()
    flipped[::3, 0], flipped[::3, 1] = tconn[::3, 1], tconn[::3, 0]  # every third tet inverted
    hconn = box.elements_nodes["hexahedron"]
    parts = [("bottom", box.node_sets["bottom"], False), ("top", box.node_sets["top"], True)]
    path = tmp_path / "box.mdpa"
    _write_mdpa(path, xyz, ids, [("Tetrahedra3D4", flipped[:20]), ("Hexahedra3D8", hconn),
                                 ("Tetrahedra3D4", flipped[20:])], parts)
    m = Mesh("mdpa_io", file_name="box.mdpa", case_dir=str(tmp_path), scale_factor=2.0)
    m.Initialize()
    np.testing.assert_allclose(m.GetNodesCoordinates(), 2.0 * xyz, rtol=0, atol=1e-15)
    assert np.array_equal(m.GetElementsNodes("hexahedron"), hconn)
    got = m.GetElementsNodes("tetra")
    assert np.array_equal(got, tconn)  # the inverted ones are swapped back (nodes 0 and 1)
    assert np.array_equal(m.GetNodeSet("bottom"), box.node_sets["bottom"])
    assert np.array_equal(m.GetNodeSet("top"), box.node_sets["top"])  # nested part skipped
    assert "inner" not in m.node_sets


def test_unknown_format_raises():
    with pytest.raises(NotImplementedError):
        Mesh("med_io", file_name="box.med", case_dir=".").Initialize()


@pytest.mark.gpu
@pytest.mark.parametrize("physics", ["thermal", "elastic", "neohooke_split"])
def test_loss_on_reference_sphere_mesh_matches_oracle(cuda, physics):
    """The reference's unstructured tetrahedral sphere: loss and both
    gradients within 1e-5 relative of the FP64 oracle."""
    from gpu_cases import gpu_loss, oracle_loss, rel_fro
    _, m = _sphere()
    # Partial_Skin_Part lies inside Skin_Part: one set per dof keeps every
    # Dirichlet dof's value unambiguous
    if physics == "thermal":
        bc = {"T": {"Partial_Skin_Part": 1.0}}
    else:
        bc = {"Ux": {"Skin_Part": 0.0}, "Uy": {"Skin_Part": 0.0}, "Uz": {"Partial_Skin_Part": 0.02}}
    s = {"dirichlet_bc_dict": bc, "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3}}
    gl, ol = gpu_loss("tet4", physics, m, s), oracle_loss("tet4", physics, m, s)
    rng = np.random.default_rng(7)
    ctrl = 0.5 + rng.random((2, gl.GetNumberOfControls()))
    u = 0.01 * rng.standard_normal((2, gl.GetTotalNumberOfDOFs()))
    a = gl.ComputeBatchLossAndGrad(ctrl, u)
    o = ol.batch_loss_and_grads(ctrl, u)
    gl.CheckDeviceStatus()
    for x, z in zip(a[2:], o[2:]):
        assert rel_fro(x.cpu().numpy(), z) < 1e-5
