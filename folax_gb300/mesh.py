"""Mesh container and structured mesh generators.

``Mesh`` mirrors the getters of fol/mesh_input_output/mesh.py:144-172 so code
written against the reference finds the same names.  The generators build
seeded, structured meshes in the reference's node/element orderings:

* create_2D_square_mesh: fol/tools/usefull_functions.py:213-258 (quad4,
  x-fastest nodes, element e = i*(N-1) + j, 'left'/'right' node sets);
* create_3D_box_mesh: structured hex8 box with the local node order of
  fol/geometries/hexahedra_3d_8.py:79-87 (the reference builds its box with
  gmsh, usefull_functions.py:187-211, which is not needed here);
* split_hex_to_tets: a conforming 6-tetrahedron split of every hexahedron,
  oriented to positive Jacobian (fol/mesh_input_output/mesh.py:123-142 swaps
  nodes 0 and 1 of negatively oriented elements; this split never needs it).

``Mesh.Initialize`` reads Kratos ``.mdpa`` files (mesh.py:93-110, 196-242):
nodes, element blocks (the Kratos geometry name mapped to the element type
key, mesh.py:15-37) and the nodes of each SubModelPart as a node set.  The
other formats the reference reads go through meshio (mesh.py:74-91), which is
not available here; they raise.
"""
from __future__ import annotations

import os

import numpy as np

# Kratos geometry names -> element type keys (the type names mesh.py:15-37 uses)
MDPA_ELEMENT_TYPES = {
    "Line2D2": "line", "Line3D2": "line", "Triangle2D3": "triangle", "Triangle3D3": "triangle",
    "Quadrilateral2D4": "quad", "Quadrilateral3D4": "quad", "Tetrahedra3D4": "tetra", "Hexahedra3D8": "hexahedron",
    "Prism3D6": "wedge", "Line2D3": "line3", "Triangle2D6": "triangle6", "Triangle3D6": "triangle6",
    "Quadrilateral2D9": "quad9", "Quadrilateral3D9": "quad9", "Tetrahedra3D10": "tetra10",
    "Hexahedra3D27": "hexahedron27", "Point2D": "vertex", "Point3D": "vertex", "Quadrilateral2D8": "quad8",
    "Quadrilateral3D8": "quad8", "Hexahedra3D20": "hexahedron20",
}


def _mdpa_element_type(block_header: str):
    """Element type of a 'Begin Elements <name>' block: the first Kratos
    geometry name contained in <name> (mesh.py:199-206 matches by substring)."""
    name = block_header[len("Begin Elements"):].strip()
    for key, etype in MDPA_ELEMENT_TYPES.items():
        if key in name:
            return etype
    return None


def read_mdpa(path: str, scale_factor: float = 1.0):
    """Parses a Kratos .mdpa file.  Returns (coordinates [N, 3],
    {element type: connectivity [E, nen]}, {SubModelPart name: node indices}).
    Node ids are mapped to 0-based row indices in file order (for the usual
    ids 1..N this is id - 1, as mesh.py:208-215 and 232-238 assume)."""
    coords, ids = [], []
    blocks: dict = {}
    sets: dict = {}
    with open(path, "r") as f:
        lines = iter(f)
        for raw in lines:
            line = raw.strip()
            if line.startswith("Begin Nodes"):
                for raw in lines:
                    t = raw.split()
                    if t and t[0] == "End":
                        break
                    if t:
                        ids.append(int(t[0]))
                        coords.append([float(t[1]), float(t[2]), float(t[3])])
            elif line.startswith("Begin Elements"):
                etype = _mdpa_element_type(line)
                rows = []
                for raw in lines:
                    t = raw.split()
                    if t and t[0] == "End":
                        break
                    if t:
                        rows.append([int(v) for v in t[2:]])  # element id, property id, node ids
                blocks.setdefault(etype, []).extend(rows)
            elif line.split()[:2] == ["Begin", "SubModelPart"]:
                # the part's own node list; nested parts are skipped
                name = line[len("Begin SubModelPart"):].strip()
                depth, node_ids = 1, None
                for raw in lines:
                    t = raw.split()
                    if t[:2] == ["Begin", "SubModelPart"]:
                        depth += 1
                    elif t[:2] == ["End", "SubModelPart"]:
                        depth -= 1
                        if depth == 0:
                            break
                    elif t[:2] == ["Begin", "SubModelPartNodes"] and depth == 1:
                        node_ids = []
                        for raw2 in lines:
                            t2 = raw2.split()
                            if t2[:1] == ["End"]:
                                break
                            if t2:
                                node_ids.append(int(t2[0]))
                if node_ids is not None:
                    sets[name] = node_ids
    index = {nid: k for k, nid in enumerate(ids)}
    xyz = scale_factor * np.asarray(coords, dtype=np.float64).reshape(-1, 3)
    conn = {et: np.asarray([[index[n] for n in row] for row in rows], dtype=np.int64) for et, rows in blocks.items()}
    node_sets = {name: np.asarray([index[n] for n in nl], dtype=np.int64) for name, nl in sets.items()}
    return xyz, conn, node_sets

ELEMENT_NODES = {"quad": 4, "hexahedron": 8, "tetra": 4}


class Mesh:
    """In-memory FE mesh (node coordinates, element connectivity, node sets)."""

    def __init__(self, io_name: str = "mesh", file_name: str = "mesh.mem", case_dir: str = ".",
                 scale_factor: float = 1.0):
        self._name = io_name
        self.file_name = file_name
        self.mesh_format = file_name.split(sep=".")[1] if "." in file_name else ""
        self.case_dir = case_dir
        self.scale_factor = scale_factor
        self.node_ids = np.zeros(0, dtype=np.int64)
        self.nodes_coordinates = np.zeros((0, 3))
        self.elements_nodes: dict[str, np.ndarray] = {}
        self.node_sets: dict[str, np.ndarray] = {}
        self.element_sets: dict[str, np.ndarray] = {}
        self.is_initialized = False

    def GetName(self) -> str:
        return self._name

    def Initialize(self) -> None:
        """Reads the mesh file (mesh.py:64-121) unless the mesh was built in
        memory ('.mem'), then orients the elements."""
        if self.is_initialized:
            return
        if self.mesh_format == "mdpa":
            xyz, conn, sets = read_mdpa(os.path.join(self.case_dir, self.file_name), self.scale_factor)
            self.nodes_coordinates = xyz
            self.node_ids = np.arange(len(xyz))
            self.elements_nodes = conn
            self.node_sets = sets
            self.element_sets = {}
        elif self.mesh_format not in ("mem", ""):
            raise NotImplementedError(f"reading .{self.mesh_format} meshes needs meshio, which is not available; "
                                      "use .mdpa or build the mesh in memory")
        self.CheckAndOrientElements()
        self.is_initialized = True

    def CheckAndOrientElements(self):
        """Swap nodes 0 and 1 of elements whose Jacobian determinant at the
        first Gauss point is negative (mesh.py:123-142)."""
        for etype, conn in self.elements_nodes.items():
            if etype not in ELEMENT_NODES:
                continue
            det = element_jacobian_det(etype, self.nodes_coordinates, conn)
            neg = det < 0
            if np.any(neg):
                conn = conn.copy()
                conn[neg, 0], conn[neg, 1] = conn[neg, 1].copy(), conn[neg, 0].copy()
                self.elements_nodes[etype] = conn

    def GetNodesIds(self):
        return self.node_ids

    def GetNumberOfNodes(self) -> int:
        return len(self.node_ids)

    def GetNodesCoordinates(self):
        return self.nodes_coordinates

    def GetNodesX(self):
        return self.nodes_coordinates[:, 0]

    def GetNodesY(self):
        return self.nodes_coordinates[:, 1]

    def GetNodesZ(self):
        return self.nodes_coordinates[:, 2]

    def GetElementsIds(self, element_type):
        return np.arange(len(self.elements_nodes[element_type]))

    def GetNumberOfElements(self, element_type) -> int:
        return len(self.elements_nodes[element_type])

    def GetElementsNodes(self, element_type):
        return self.elements_nodes[element_type]

    def GetNodeSet(self, set_name):
        return self.node_sets[set_name]


def element_jacobian_det(etype: str, xyz: np.ndarray, conn: np.ndarray) -> np.ndarray:
    """det J at the element's first-order Gauss point (centre / (1/4,1/4,1/4))."""
    X = xyz[conn]
    if etype == "tetra":
        J = np.stack([X[:, 1] - X[:, 0], X[:, 2] - X[:, 0], X[:, 3] - X[:, 0]], axis=2)
        return np.linalg.det(J)
    if etype == "quad":
        d = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], dtype=float) * 0.25
        J = np.einsum("eai,ak->eik", X[:, :, :2], d)
        return np.linalg.det(J)
    s = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                  [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=float) * 0.125
    J = np.einsum("eai,ak->eik", X, s)
    return np.linalg.det(J)


def create_2D_square_mesh(L: float, N: int) -> Mesh:
    """Structured quad4 mesh of (N-1)^2 elements on [0,L]^2 (usefull_functions.py:213-258)."""
    mesh = Mesh("square_io", "square.mem")
    Ne = N - 1
    x = np.linspace(0.0, L, N)
    X, Y = np.meshgrid(x, x)
    mesh.node_ids = np.arange(N * N)
    mesh.nodes_coordinates = np.stack([X.ravel(), Y.ravel(), np.zeros(N * N)], axis=1)
    i, j = np.meshgrid(np.arange(Ne), np.arange(Ne), indexing="ij")
    i, j = i.ravel(), j.ravel()
    conn = np.stack([i * N + j, i * N + j + 1, (i + 1) * N + j + 1, (i + 1) * N + j], axis=1)
    mesh.elements_nodes = {"quad": conn.astype(np.int64)}
    mesh.node_sets = {"left": np.arange(0, N * N, N), "right": np.arange(N - 1, N * N, N),
                      "bottom": np.arange(0, N), "top": np.arange(N * (N - 1), N * N)}
    mesh.is_initialized = True
    return mesh


def create_3D_box_mesh(Nx: int, Ny: int, Nz: int, Lx: float = 1.0, Ly: float = 1.0, Lz: float = 1.0) -> Mesh:
    """Structured hex8 box of Nx*Ny*Nz elements; nodes x-fastest, then y, then z.

    Node sets: left/right (x = 0 / Lx), front/back (y = 0 / Ly),
    bottom/top (z = 0 / Lz).  Element e = (k*Ny + j)*Nx + i.
    """
    mesh = Mesh("box_io", "box.mem")
    nx, ny, nz = Nx + 1, Ny + 1, Nz + 1
    xs, ys, zs = np.linspace(0, Lx, nx), np.linspace(0, Ly, ny), np.linspace(0, Lz, nz)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    mesh.nodes_coordinates = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    mesh.node_ids = np.arange(nx * ny * nz)
    k, j, i = np.meshgrid(np.arange(Nz), np.arange(Ny), np.arange(Nx), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()

    def nid(ii, jj, kk):
        return (kk * ny + jj) * nx + ii

    conn = np.stack([nid(i, j, k), nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i, j + 1, k),
                     nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1)],
                    axis=1)
    mesh.elements_nodes = {"hexahedron": conn.astype(np.int64)}
    ids = mesh.node_ids.reshape(nz, ny, nx)
    mesh.node_sets = {"left": ids[:, :, 0].ravel(), "right": ids[:, :, -1].ravel(),
                      "front": ids[:, 0, :].ravel(), "back": ids[:, -1, :].ravel(),
                      "bottom": ids[0].ravel(), "top": ids[-1].ravel()}
    mesh.is_initialized = True
    return mesh


# Kuhn split of the unit cube along the diagonal from local node 0 (-,-,-) to
# local node 6 (+,+,+): one tetrahedron per axis permutation.  Local hex nodes:
# 0 (000) 1 (100) 2 (110) 3 (010) 4 (001) 5 (101) 6 (111) 7 (011).
_KUHN = np.array([[0, 1, 2, 6], [0, 2, 3, 6], [0, 3, 7, 6], [0, 7, 4, 6], [0, 4, 5, 6], [0, 5, 1, 6]])


def split_hex_to_tets(hex_mesh: Mesh) -> Mesh:
    """Conforming 6-tet split of every hexahedron (6*E tetrahedra)."""
    conn = hex_mesh.elements_nodes["hexahedron"]
    tets = conn[:, _KUHN].reshape(-1, 4)
    det = element_jacobian_det("tetra", hex_mesh.nodes_coordinates, tets)
    neg = det < 0
    tets[neg, 1], tets[neg, 2] = tets[neg, 2].copy(), tets[neg, 1].copy()
    mesh = Mesh("tet_io", "tets.mem")
    mesh.node_ids = hex_mesh.node_ids.copy()
    mesh.nodes_coordinates = hex_mesh.nodes_coordinates.copy()
    mesh.elements_nodes = {"tetra": tets.astype(np.int64)}
    mesh.node_sets = {k: v.copy() for k, v in hex_mesh.node_sets.items()}
    mesh.is_initialized = True
    return mesh
