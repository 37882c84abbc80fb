"""folax_gb300 — GB300 (sm_103a) finite-element weighted-residual hot path.

The package keeps the reference's FiniteElementLoss / Solver API
(fol/loss_functions, fol/solvers) and runs every numerical step in the CUDA
kernels of libfolgb.so (C ABI: include/folgb.h).  Loss classes live in
``folax_gb300.loss`` (the split neo-Hooke family of the reference's
mechanical_neohooke.py in ``folax_gb300.mechanical_neohooke``), solvers in
``folax_gb300.solvers``, the many-instance path in ``folax_gb300.batched``.
"""
from .mesh import Mesh, create_2D_square_mesh, create_3D_box_mesh, split_hex_to_tets  # noqa: F401

_LAZY = {
    "loss": ("FiniteElementLoss", "ThermalLoss2DQuad", "ThermalLoss3DHexa", "ThermalLoss3DTetra",
             "MechanicalLoss2DQuad", "MechanicalLoss3DHexa", "MechanicalLoss3DTetra",
             "NeoHookeMechanicalLoss2DQuad", "NeoHookeMechanicalLoss3DHexa", "NeoHookeMechanicalLoss3DTetra",
             "SaintVenantMechanicalLoss2DQuad", "SaintVenantMechanicalLoss3DHexa", "SaintVenantMechanicalLoss3DTetra"),
    "solvers": ("FiniteElementLinearResidualBasedSolver", "FiniteElementNonLinearResidualBasedSolver"),
}


def __getattr__(name):
    import importlib
    for mod, names in _LAZY.items():
        if name in names:
            return getattr(importlib.import_module(f"{__name__}.{mod}"), name)
    raise AttributeError(name)
