"""Seeded synthetic workloads of the benchmark configurations.

Each builder returns the mesh, the loss settings in the reference's keys and
the seeded inputs of one configuration, so the benchmark and the full-size
parity tests evaluate exactly the same problems.  Fields come from
folax_gb300.fields (numpy.random.default_rng; the seeds are arguments).

* square_thermal     quad4 steady heat conduction on the unit square, n x n
                     elements, per-element Fourier conductivity, T = 1 at
                     x = 0 and T = 0 at x = 1 (plain method, small).
* hex8_elastic       hex8 linear elasticity on the unit cube, n^3 elements,
                     two-phase voxel Young's modulus per element, u = 0 on
                     z = 0, u_z = 0.05 on z = 1; dofs = the uniaxial field
                     u_z = 0.05 z plus N(0, 0.01^2) noise.
* thermal_instances  many quad4 thermal squares, sides n ~ U{16..128}, each
                     with its own Fourier conductivity.
* neohooke_tets      the 6-tet split of an n^3 hex grid, neo-Hookean (AD),
                     one two-phase field per instance (seed + i), dofs =
                     uniaxial field plus N(0, (0.01 h)^2) noise per instance
                     (h = 1/n: displacement-gradient noise of about 0.01, so
                     every tet keeps det F > 0 and the log terms stay finite).
"""
from __future__ import annotations

import numpy as np

from . import fields
from .mesh import create_2D_square_mesh, create_3D_box_mesh, split_hex_to_tets

UNIAXIAL_BC = {"Ux": {"bottom": 0.0}, "Uy": {"bottom": 0.0}, "Uz": {"bottom": 0.0, "top": 0.05}}
THERMAL_BC = {"T": {"left": 1.0, "right": 0.0}}


def square_thermal(n: int = 50, seed: int = 5):
    """(mesh, settings, k per element)."""
    m = create_2D_square_mesh(1.0, n + 1)
    k = fields.fourier_conductivity(fields.element_centroids(m.nodes_coordinates, m.elements_nodes["quad"]), seed)
    settings = {"dirichlet_bc_dict": dict(THERMAL_BC), "control_layout": "element", "num_gp": 2}
    return m, settings, k


def hex8_elastic(n: int = 64, seed: int = 2024, jitter: float = 0.0):
    """(mesh, settings, E per element float32, dofs float32).  jitter > 0
    moves every interior node by N(0, (jitter h)^2) per coordinate (h = 1/n,
    boundary nodes stay on their faces), so no element is a parallelepiped."""
    mesh = create_3D_box_mesh(n, n, n)
    if jitter > 0.0:
        rng_x = np.random.default_rng(seed + 7)
        x = mesh.nodes_coordinates
        d = (jitter / n) * rng_x.standard_normal(x.shape)
        on_face = (np.abs(x) < 1e-12) | (np.abs(x - 1.0) < 1e-12)
        d[on_face] = 0.0
        mesh.nodes_coordinates = x + d
    E = fields.two_phase_voxels(n, seed, sigma=3.0, high=1.0, low=0.1)
    rng = np.random.default_rng(seed + 1)
    u = np.zeros((mesh.GetNumberOfNodes(), 3))
    u[:, 2] = 0.05 * mesh.nodes_coordinates[:, 2]
    u += 0.01 * rng.standard_normal(u.shape)
    settings = {"dirichlet_bc_dict": {k: dict(v) for k, v in UNIAXIAL_BC.items()},
                "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3},
                "control_layout": "element", "num_gp": 2}
    return mesh, settings, E.astype(np.float32), u.ravel().astype(np.float32)


def thermal_instances(n_inst: int = 512, seed: int = 11):
    """(meshes, settings, per-instance conductivity arrays)."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(16, 129, n_inst)
    meshes = [create_2D_square_mesh(1.0, int(n) + 1) for n in sizes]
    settings = {"dirichlet_bc_dict": dict(THERMAL_BC), "control_layout": "element", "num_gp": 2}
    ks = [fields.fourier_conductivity(fields.element_centroids(m.nodes_coordinates, m.elements_nodes["quad"]), seed + i)
          for i, m in enumerate(meshes)]
    return meshes, settings, ks


def neohooke_tets(n: int = 64, batch: int = 16, seed: int = 2024):
    """(mesh, settings, E [batch, tets] float32, dofs [batch, dofs] float32):
    instance i has the two-phase field of seed + i (one value per hex cell,
    repeated over its 6 tets)."""
    mesh = split_hex_to_tets(create_3D_box_mesh(n, n, n))
    E = np.stack([np.repeat(fields.two_phase_voxels(n, seed + i), 6) for i in range(batch)]).astype(np.float32)
    settings = {"dirichlet_bc_dict": {k: dict(v) for k, v in UNIAXIAL_BC.items()},
                "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3}, "control_layout": "element"}
    rng = np.random.default_rng(seed)
    u = np.zeros((batch, mesh.GetNumberOfNodes(), 3), dtype=np.float32)
    u[:, :, 2] = 0.05 * mesh.nodes_coordinates[None, :, 2]
    u += ((0.01 / n) * rng.standard_normal(u.shape)).astype(np.float32)
    return mesh, settings, E, u.reshape(batch, -1)
