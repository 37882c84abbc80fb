"""Shared builders for the GPU parity tests: the same seeded mesh, settings
and fields go to the GPU loss classes and to the FP64 oracle."""
import numpy as np

from folax_gb300 import mesh as M
from oracle import fe_oracle as fo

ETYPE_NAME = {"quad4": "quad", "hex8": "hexahedron", "tet4": "tetra"}


def make_mesh(etype, n, seed=0, jitter=0.08):
    """Structured mesh with nodes displaced by N(0, (jitter * h)^2), h = 1/n."""
    rng = np.random.default_rng(seed)
    amp = jitter / n
    if etype == "quad4":
        m = M.create_2D_square_mesh(1.0, n + 1)
        m.nodes_coordinates = m.nodes_coordinates + amp * rng.standard_normal(m.nodes_coordinates.shape) * np.array([1, 1, 0])
    else:
        m = M.create_3D_box_mesh(n, n, n)
        m.nodes_coordinates = m.nodes_coordinates + amp * rng.standard_normal(m.nodes_coordinates.shape)
        if etype == "tet4":
            m = M.split_hex_to_tets(m)
    return m


def bc_dict(etype, physics, nonzero=True):
    v = 1.0 if nonzero else 0.0
    w = 0.05 if nonzero else 0.0
    if physics == "thermal":
        return {"T": {"left": v, "right": 0.0}} if etype == "quad4" else {"T": {"bottom": v, "top": 0.0}}
    if etype == "quad4":
        return {"Ux": {"left": 0.0, "right": w}, "Uy": {"left": 0.0}}
    return {"Ux": {"bottom": 0.0}, "Uy": {"bottom": 0.0}, "Uz": {"bottom": 0.0, "top": w}}


def gpu_loss(etype, physics, m, settings):
    from folax_gb300 import loss as L
    from folax_gb300 import mechanical_neohooke as NH
    cls = {("quad4", "thermal"): L.ThermalLoss2DQuad, ("hex8", "thermal"): L.ThermalLoss3DHexa,
           ("tet4", "thermal"): L.ThermalLoss3DTetra, ("quad4", "elastic"): L.MechanicalLoss2DQuad,
           ("hex8", "elastic"): L.MechanicalLoss3DHexa, ("tet4", "elastic"): L.MechanicalLoss3DTetra,
           ("quad4", "neohooke"): L.NeoHookeMechanicalLoss2DQuad, ("hex8", "neohooke"): L.NeoHookeMechanicalLoss3DHexa,
           ("tet4", "neohooke"): L.NeoHookeMechanicalLoss3DTetra,
           ("quad4", "saint_venant"): L.SaintVenantMechanicalLoss2DQuad,
           ("hex8", "saint_venant"): L.SaintVenantMechanicalLoss3DHexa,
           ("tet4", "saint_venant"): L.SaintVenantMechanicalLoss3DTetra,
           ("quad4", "neohooke_split"): NH.NeoHookeMechanicalLoss2DQuad,
           ("hex8", "neohooke_split"): NH.NeoHookeMechanicalLoss3DHexa,
           ("tet4", "neohooke_split"): NH.NeoHookeMechanicalLoss3DTetra}[(etype, physics)]
    loss = cls("loss", dict(settings), m)
    loss.Initialize()
    return loss


def oracle_loss(etype, physics, m, settings):
    mat = settings.get("material_dict", {})
    return fo.FELossOracle(etype, physics, m.nodes_coordinates, m.elements_nodes[ETYPE_NAME[etype]],
                           dirichlet=settings["dirichlet_bc_dict"], node_sets=m.node_sets,
                           num_gp=settings.get("num_gp", 1 if etype == "tet4" else 2),
                           young=mat.get("young_modulus", 1.0), nu=mat.get("poisson_ratio", 0.3),
                           body_force=settings.get("body_foce"), beta=settings.get("beta", 0.0),
                           c=settings.get("c", 1.0), exponent=settings.get("loss_function_exponent", 1.0),
                           shear_mode=settings.get("voigt_shear_mode", "reference"),
                           control_layout=settings.get("control_layout", "nodal"))


def rel_fro(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


def c_oracle_loss(etype, physics, m, settings):
    """The C FP64 oracle (thermal / elastic) with the same arguments."""
    from oracle import c_oracle
    mat = settings.get("material_dict", {})
    return c_oracle.CLossOracle(etype, physics, m.nodes_coordinates, m.elements_nodes[ETYPE_NAME[etype]],
                                dirichlet=settings["dirichlet_bc_dict"], node_sets=m.node_sets,
                                num_gp=settings.get("num_gp", 1 if etype == "tet4" else 2),
                                young=mat.get("young_modulus", 1.0), nu=mat.get("poisson_ratio", 0.3),
                                body_force=settings.get("body_foce"), beta=settings.get("beta", 0.0),
                                c=settings.get("c", 1.0), exponent=settings.get("loss_function_exponent", 1.0),
                                control_layout=settings.get("control_layout", "nodal"))
