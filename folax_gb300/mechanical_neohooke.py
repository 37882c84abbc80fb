"""Neo-Hookean elements with a volumetric-isochoric split, the non-AD element
family of fol/loss_functions/mechanical_neohooke.py (the module of that name
in the reference, beside mechanical_neohooke_AD.py whose classes carry the
same names; those live in ``folax_gb300.loss``).

Per Gauss point kappa = E/(3(1-2 nu)) and mu = E/(2(1+nu)) from the
interpolated Young's modulus control (mechanical_neohooke.py:253-255),
psi = kappa/4 (J^2 - 2 ln J - 1) + mu/2 (J^(-2/d) I1 - d) and its
S = 2 dpsi/dC (constitutive_material_models/neo_hooke.py:14-111).  Energy
sum w detJ psi (the loss), residual B(F)^T S - Fe, tangent B^T C B plus the
geometric stiffness (:243-275); the tangent is the exact derivative of the
residual, so the loss gradient with respect to the dofs is the internal
force.  Every number comes from the CUDA kernels of libfolgb.so.
"""
from __future__ import annotations

from . import _capi as capi
from .loss import FiniteElementLoss, _with


class NeoHookeMechanicalLoss(FiniteElementLoss):
    """mechanical_neohooke.py:16-275 over the GB300 kernels."""
    physics = capi.NEOHOOKE_SPLIT

    def Initialize(self, reinitialize=False) -> None:
        if "material_dict" not in self.loss_settings:
            raise ValueError("material_dict should provided in the loss settings !")
        super().Initialize(reinitialize)


class NeoHookeMechanicalLoss3DTetra(NeoHookeMechanicalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        super().__init__(name, _with(loss_settings, compute_dims=3, ordered_dofs=["Ux", "Uy", "Uz"],
                                     element_type="tetra"), fe_mesh)


class NeoHookeMechanicalLoss3DHexa(NeoHookeMechanicalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        loss_settings.setdefault("num_gp", 2)
        super().__init__(name, _with(loss_settings, compute_dims=3, ordered_dofs=["Ux", "Uy", "Uz"],
                                     element_type="hexahedron"), fe_mesh)


class NeoHookeMechanicalLoss2DQuad(NeoHookeMechanicalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        loss_settings.setdefault("num_gp", 2)
        super().__init__(name, _with(loss_settings, compute_dims=2, ordered_dofs=["Ux", "Uy"], element_type="quad"),
                         fe_mesh)
