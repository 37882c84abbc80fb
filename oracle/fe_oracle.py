"""FP64 NumPy restatement of folax's finite-element weighted-residual path.

TEST INFRASTRUCTURE ONLY.  This module is the correctness oracle: it is imported
by ``tests/``, by ``__graft_entry__.smoke()`` as the checker, and by
``bench.py``'s CPU-baseline leg.  The product path (``folax_gb300``) never
imports it.

Parity is pinned: ``tests/test_oracle_golden.py`` checks this module against the
reference's own golden vectors (``tests/golden/*.json``, extracted from the
reference's unit tests by ``tests/golden/make_golden.py``).

Every function cites the reference file:line it restates (paths are relative
to the folax project root).  All arithmetic is float64 (or complex128 when a
caller uses the complex-step trick to differentiate through it).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

# ----------------------------------------------------------------------------
# Geometry: shape functions and Gauss rules
#   fol/geometries/quadrilateral_2d_4.py:16-70, hexahedra_3d_8.py:16-114,
#   tetrahedra_3d_4.py:16-60, geometry.py:87-97
# ----------------------------------------------------------------------------

ELEMENTS = {
    # name: (nodes per element, reference-space dimension)
    "quad4": (4, 2),
    "hex8": (8, 3),
    "tet4": (4, 3),
}

# local node sign pattern of the trilinear hexahedron (hexahedra_3d_8.py:79-87)
_HEX_SIGNS = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                       [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=np.float64)
# local node sign pattern of the bilinear quadrilateral (quadrilateral_2d_4.py:61-65)
_QUAD_SIGNS = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], dtype=np.float64)

# Keast-type 8-point tetrahedron rule used by the reference for order 3
# (tetrahedra_3d_4.py:36-48): two orbits of four points.
_TET3_A = (0.015835909865720057993, 0.32805469671142664734, 0.02308799441864369039)
_TET3_B = (0.67914317820120795168, 0.10695227393293068277, 0.01857867224802297628)


def _gauss_1d(order):
    if order == 1:
        return np.array([0.0]), np.array([2.0])
    if order == 2:
        g = 1.0 / math.sqrt(3.0)
        return np.array([-g, g]), np.array([1.0, 1.0])
    if order == 3:
        a = math.sqrt(3.0 / 5.0)
        return np.array([-a, 0.0, a]), np.array([5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0])
    raise NotImplementedError(f"Gauss order {order} is not implemented")


def gauss_rule(etype: str, order: int):
    """Integration points (n, 3) and weights (n,) in the reference's point order.

    quad4/hex8 order 2 follow the node sign ordering (quadrilateral_2d_4.py:24-30,
    hexahedra_3d_8.py:22-33); order 1 and 3 are tensor products with the first
    coordinate running fastest (quadrilateral_2d_4.py:33-45, hexahedra_3d_8.py:36-70).
    """
    if order not in (1, 2, 3):
        raise NotImplementedError(f"{etype}: Gauss order {order} is not implemented")
    if etype == "tet4":
        if order == 1:
            return np.array([[0.25, 0.25, 0.25]]), np.array([1.0 / 6.0])
        if order == 2:
            a, b = 0.58541020, 0.13819660
            pts = np.array([[a, b, b], [b, a, b], [b, b, a], [b, b, b]])
            return pts, np.full(4, 1.0 / 24.0)
        pts, wts = [], []
        for lo, hi, w in (_TET3_A, _TET3_B):
            pts += [[lo, hi, hi], [hi, lo, hi], [hi, hi, lo], [hi, hi, hi]]
            wts += [w] * 4
        return np.array(pts), np.array(wts)
    nen, dim = ELEMENTS[etype]
    g, w = _gauss_1d(order)
    if order == 2:
        signs = _QUAD_SIGNS if etype == "quad4" else _HEX_SIGNS
        pts = signs * g[1]
        wts = np.ones(len(signs))
    else:
        grids = np.meshgrid(*([g] * dim), indexing="ij")
        wgrid = np.meshgrid(*([w] * dim), indexing="ij")
        # first coordinate fastest
        pts = np.stack([gr.transpose().ravel() for gr in grids], axis=1)
        wts = np.prod(np.stack([wg.transpose().ravel() for wg in wgrid], axis=1), axis=1)
    if dim == 2:
        pts = np.concatenate([pts, np.zeros((len(pts), 1))], axis=1)
    return pts, wts


def shape_values(etype: str, xi):
    """N_a(xi) (nen,)."""
    xi = np.asarray(xi)
    if etype == "tet4":
        return np.array([1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]])
    if etype == "quad4":
        s = _QUAD_SIGNS
        return 0.25 * (1 + s[:, 0] * xi[0]) * (1 + s[:, 1] * xi[1])
    s = _HEX_SIGNS
    return 0.125 * (1 + s[:, 0] * xi[0]) * (1 + s[:, 1] * xi[1]) * (1 + s[:, 2] * xi[2])


def shape_local_grads(etype: str, xi):
    """dN_a/dxi_k (nen, dim)."""
    xi = np.asarray(xi)
    if etype == "tet4":
        return np.array([[-1.0, -1.0, -1.0], [1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0]])
    if etype == "quad4":
        s = _QUAD_SIGNS
        return np.stack([0.25 * s[:, 0] * (1 + s[:, 1] * xi[1]),
                         0.25 * s[:, 1] * (1 + s[:, 0] * xi[0])], axis=1)
    s = _HEX_SIGNS
    f = 1 + s * xi[:3]
    return 0.125 * np.stack([s[:, 0] * f[:, 1] * f[:, 2],
                             s[:, 1] * f[:, 0] * f[:, 2],
                             s[:, 2] * f[:, 0] * f[:, 1]], axis=1)


def _det(J):
    d = J.shape[-1]
    if d == 2:
        return J[..., 0, 0] * J[..., 1, 1] - J[..., 0, 1] * J[..., 1, 0]
    return (J[..., 0, 0] * (J[..., 1, 1] * J[..., 2, 2] - J[..., 1, 2] * J[..., 2, 1])
            - J[..., 0, 1] * (J[..., 1, 0] * J[..., 2, 2] - J[..., 1, 2] * J[..., 2, 0])
            + J[..., 0, 2] * (J[..., 1, 0] * J[..., 2, 1] - J[..., 1, 1] * J[..., 2, 0]))


def _inv(J):
    return np.linalg.inv(J)


def jacobian(etype: str, X, xi):
    """J[i,k] = sum_a X[a,i] dN_a/dxi_k  (geometry.py:93-97; quad4 uses x,y only,
    quadrilateral_2d_4.py:67-70).  X: (..., nen, 3)."""
    nen, dim = ELEMENTS[etype]
    dN = shape_local_grads(etype, xi)
    return np.einsum("...ai,ak->...ik", X[..., :dim], dN)


def global_grads(etype: str, X, xi):
    """dN_a/dx_j = dN_a/dxi_k (J^-1)_kj, plus detJ (geometry.py:87-91)."""
    J = jacobian(etype, X, xi)
    dN = shape_local_grads(etype, xi)
    return np.einsum("ak,...kj->...aj", dN, _inv(J)), _det(J)


# ----------------------------------------------------------------------------
# Element physics
# ----------------------------------------------------------------------------

def isotropic_D(dim, young, nu):
    """Constitutive matrix: 3-D isotropic (mechanical.py:63-82) or 2-D plane
    stress (mechanical.py:60-61)."""
    if dim == 2:
        return np.array([[1, nu, 0], [nu, 1, 0], [0, 0, (1 - nu) / 2]]) * (young / (1 - nu ** 2))
    c1 = young / ((1.0 + nu) * (1.0 - 2.0 * nu))
    c2, c3, c4 = c1 * (1.0 - nu), c1 * nu, c1 * 0.5 * (1.0 - 2.0 * nu)
    D = np.zeros((6, 6))
    D[:3, :3] = c3
    D[0, 0] = D[1, 1] = D[2, 2] = c2
    D[3, 3] = D[4, 4] = D[5, 5] = c4
    return D


def small_strain_B(dNdx):
    """Small-strain B (..., nvoigt, dim*nen) in the reference's row order
    (mechanical.py:35-58: 3-D rows xx,yy,zz,xy,yz,xz; 2-D rows xx,yy,xy)."""
    nen, dim = dNdx.shape[-2:]
    shp = dNdx.shape[:-2]
    if dim == 2:
        B = np.zeros(shp + (3, 2 * nen), dtype=dNdx.dtype)
        B[..., 0, 0::2] = dNdx[..., 0]
        B[..., 1, 1::2] = dNdx[..., 1]
        B[..., 2, 0::2] = dNdx[..., 1]
        B[..., 2, 1::2] = dNdx[..., 0]
        return B
    B = np.zeros(shp + (6, 3 * nen), dtype=dNdx.dtype)
    B[..., 0, 0::3] = dNdx[..., 0]
    B[..., 1, 1::3] = dNdx[..., 1]
    B[..., 2, 2::3] = dNdx[..., 2]
    B[..., 3, 0::3] = dNdx[..., 1]
    B[..., 3, 1::3] = dNdx[..., 0]
    B[..., 4, 1::3] = dNdx[..., 2]
    B[..., 4, 2::3] = dNdx[..., 1]
    B[..., 5, 0::3] = dNdx[..., 2]
    B[..., 5, 2::3] = dNdx[..., 0]
    return B


def N_matrix(Nv, ndof):
    """Interleaved shape-function matrix (ndof, ndof*nen) (mechanical.py:84-96)."""
    nen = Nv.shape[-1]
    M = np.zeros((ndof, ndof * nen), dtype=Nv.dtype)
    for c in range(ndof):
        M[c, c::ndof] = Nv
    return M


def _as_batch(X, de, ue):
    X = np.asarray(X)
    squeeze = X.ndim == 2
    if squeeze:
        X = X[None]
        de = np.asarray(de)[None]
        ue = np.asarray(ue)[None]
    return X, np.asarray(de), np.asarray(ue), squeeze


def thermal_element(etype, X, de, te, num_gp=2, beta=0.0, c=1.0, body_force=0.0):
    """Thermal element (thermal.py:28-49).  Returns (energy, re, Se, dEnergy/dde).

    X (E, nen, 3), de (E, nen) nodal conductivity controls, te (E, nen).
    energy = te . stop_gradient(Se te - Fe); the control derivative is the true
    derivative of the energy VALUE (the reference's jax.grad wrt de is 0 there).
    """
    X, de, te, squeeze = _as_batch(X, de, te)
    nen, dim = ELEMENTS[etype]
    pts, wts = gauss_rule(etype, num_gp)
    E = X.shape[0]
    dt = np.result_type(X, de, te)
    Se = np.zeros((E, nen, nen), dtype=dt)
    Fe = np.zeros((E, nen), dtype=dt)
    dEn = np.zeros((E, nen), dtype=dt)
    for xi, w in zip(pts, wts):
        Nv = shape_values(etype, xi)
        dNdx, detJ = global_grads(etype, X, xi)
        g = 1.0 + beta * (te @ Nv) ** c
        k = (de @ Nv) * g
        wd = w * detJ
        Se += (wd * k)[:, None, None] * np.einsum("eaj,ebj->eab", dNdx, dNdx)
        Fe += (wd * body_force)[:, None] * Nv[None]
        gradT = np.einsum("ea,eaj->ej", te, dNdx)
        dEn += (wd * g * np.einsum("ej,ej->e", gradT, gradT))[:, None] * Nv[None]
    re = np.einsum("eab,eb->ea", Se, te) - Fe
    energy = np.einsum("ea,ea->e", te, re)
    if squeeze:
        return energy[0], re[0], Se[0], dEn[0]
    return energy, re, Se, dEn


def linear_elastic_element(etype, X, de, ue, num_gp=2, young=1.0, nu=0.3, body_force=None):
    """Small-strain elastic element (mechanical.py:98-117).

    Returns (energy, re, Se, dEnergy/dde) with energy = ue . stop_gradient(Se ue - Fe),
    Se = sum_gp w detJ (N.de) B^T D B, Fe = sum_gp w detJ N^T b.
    """
    X, de, ue, squeeze = _as_batch(X, de, ue)
    nen, dim = ELEMENTS[etype]
    ndof = dim
    D = isotropic_D(dim, young, nu)
    b = np.zeros(dim) if body_force is None else np.asarray(body_force, dtype=np.float64).ravel()[:dim]
    pts, wts = gauss_rule(etype, num_gp)
    E = X.shape[0]
    dt = np.result_type(X, de, ue)
    Se = np.zeros((E, ndof * nen, ndof * nen), dtype=dt)
    Fe = np.zeros((E, ndof * nen), dtype=dt)
    dEn = np.zeros((E, nen), dtype=dt)
    for xi, w in zip(pts, wts):
        Nv = shape_values(etype, xi)
        dNdx, detJ = global_grads(etype, X, xi)
        B = small_strain_B(dNdx)
        egp = de @ Nv
        wd = w * detJ
        BtDB = np.einsum("evi,vw,ewj->eij", B, D, B)
        Se += (wd * egp)[:, None, None] * BtDB
        Fe += wd[:, None] * (N_matrix(Nv, ndof).T @ b)[None]
        eps = np.einsum("evi,ei->ev", B, ue)
        dEn += (wd * np.einsum("ev,vw,ew->e", eps, D, eps))[:, None] * Nv[None]
    re = np.einsum("eij,ej->ei", Se, ue) - Fe
    energy = np.einsum("ei,ei->e", ue, re)
    if squeeze:
        return energy[0], re[0], Se[0], dEn[0]
    return energy, re, Se, dEn


# --- Neo-Hookean (AD variant) -------------------------------------------------
# fol/loss_functions/mechanical_neohooke_AD.py:52-95, 254-293;
# fol/constitutive_material_models/neo_hooke.py:112-157 (3-D), 159-201 (2-D);
# Voigt conventions fol/constitutive_material_models/utils.py:13-56.

_V3 = [(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]   # [xx,yy,zz,yz,xz,xy]
_V2 = [(0, 0), (1, 1), (0, 1)]                           # [xx,yy,xy]


def lame(e, nu):
    """mu, lambda from the Young's modulus field at a Gauss point
    (mechanical_neohooke_AD.py:264-267)."""
    return e / (2.0 * (1.0 + nu)), e * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))


def nh_energy_stress(C, mu, lam):
    """Strain energy psi(C), true second Piola-Kirchhoff S(C), and its
    directional-derivative operator.  3-D: psi = mu/2 (J^-2/3 I1 - 3) - mu lnJ
    + lam/2 ln^2 J (neo_hooke.py:129-135); 2-D: psi = mu/2 (I1 - 2) - mu lnJ
    + lam/2 ln^2 J (neo_hooke.py:178-181).  C: (..., d, d)."""
    d = C.shape[-1]
    detC = _det(C)
    lnJ = 0.5 * np.log(detC)
    Ci = _inv(C)
    I1 = np.trace(C, axis1=-2, axis2=-1)
    eye = np.eye(d)
    mu_ = mu[..., None, None]
    lam_ = lam[..., None, None]
    if d == 3:
        a = np.exp(-2.0 / 3.0 * lnJ)           # J^(-2/3)
        psi = 0.5 * mu * (a * I1 - 3.0) - mu * lnJ + 0.5 * lam * lnJ ** 2
        S = (mu_ * a[..., None, None] * (eye - (I1 / 3.0)[..., None, None] * Ci)
             + (lam_ * lnJ[..., None, None] - mu_) * Ci)
        dpsi_dmu = 0.5 * (a * I1 - 3.0) - lnJ
    else:
        a = None
        psi = 0.5 * mu * (I1 - 2.0) - mu * lnJ + 0.5 * lam * lnJ ** 2
        S = mu_ * (eye - Ci) + lam_ * lnJ[..., None, None] * Ci
        dpsi_dmu = 0.5 * (I1 - 2.0) - lnJ
    dpsi_dlam = 0.5 * lnJ ** 2

    def dS(dC):
        """Directional derivative of S along a symmetric dC (..., d, d)."""
        trCidC = np.einsum("...ij,...ji->...", Ci, dC)
        dCi = -Ci @ dC @ Ci
        dlnJ = 0.5 * trCidC
        out = (lam_ * dlnJ[..., None, None]) * Ci + (lam_ * lnJ[..., None, None] - mu_) * dCi
        if d == 3:
            da = -(1.0 / 3.0) * a * trCidC
            dI1 = np.trace(dC, axis1=-2, axis2=-1)
            out = out + mu_ * (da[..., None, None] * (eye - (I1 / 3.0)[..., None, None] * Ci)
                               - a[..., None, None] * ((dI1 / 3.0)[..., None, None] * Ci
                                                       + (I1 / 3.0)[..., None, None] * dCi))
        return out

    return psi, S, dS, dpsi_dmu, dpsi_dlam


def nl_B(F, dNdx):
    """Green-Lagrange B(F) (..., nvoigt, d*nen) of CalculateKinematics3D/2D
    (mechanical_neohooke_AD.py:52-95): row v, column d*a+k = dE_v/du_{a,k} with
    engineering shear rows."""
    nen, d = dNdx.shape[-2:]
    V = _V3 if d == 3 else _V2
    B = np.zeros(F.shape[:-2] + (len(V), d * nen), dtype=np.result_type(F, dNdx))
    for v, (p, q) in enumerate(V):
        for k in range(d):
            if p == q:
                B[..., v, k::d] = F[..., k, p, None] * dNdx[..., p]
            else:
                B[..., v, k::d] = F[..., k, p, None] * dNdx[..., q] + F[..., k, q, None] * dNdx[..., p]
    return B


def neohooke_element(etype, X, de, ue, num_gp=None, nu=0.3, body_force=None,
                     shear_mode="reference", want_tangent=True):
    """Neo-Hookean AD element (mechanical_neohooke_AD.py:254-293).

    Returns (energy, re, Ke, fint_consistent, dEnergy/dde):
      energy = sum_gp w detJ psi                                         (:284,:292)
      re     = sum_gp w detJ B^T S_voigt - Fe, with S_voigt = 2 dpsi/dC_voigt;
               the reference's VoigtToTensor fills both off-diagonal slots, so
               its shear entries are 2 S_ij ("reference" mode, utils.py:45-56);
               "consistent" mode uses S_ij (the true energy gradient).
      Ke     = d re / d ue (jacfwd of the residual, :275,:281), same mode as re.
      fint_consistent = sum_gp w detJ B^T S (consistent) = d energy / d ue.
    """
    X, de, ue, squeeze = _as_batch(X, de, ue)
    nen, d = ELEMENTS[etype]
    if num_gp is None:
        num_gp = 1 if etype == "tet4" else 2
    V = _V3 if d == 3 else _V2
    m_ref = np.array([1.0 if p == q else 2.0 for p, q in V])
    m_use = m_ref if shear_mode == "reference" else np.ones(len(V))
    b = np.zeros(d) if body_force is None else np.asarray(body_force, dtype=np.float64).ravel()[:d]
    pts, wts = gauss_rule(etype, num_gp)
    E = X.shape[0]
    dt = np.result_type(X, de, ue)
    nd = d * nen
    energy = np.zeros(E, dtype=dt)
    fint = np.zeros((E, nd), dtype=dt)
    fcons = np.zeros((E, nd), dtype=dt)
    Fe = np.zeros((E, nd), dtype=dt)
    Ke = np.zeros((E, nd, nd), dtype=dt) if want_tangent else None
    dEn = np.zeros((E, nen), dtype=dt)
    U = ue.reshape(E, nen, d)
    for xi, w in zip(pts, wts):
        Nv = shape_values(etype, xi)
        dNdx, detJ = global_grads(etype, X, xi)
        wd = w * detJ
        egp = de @ Nv
        mu, lam = lame(egp, nu)
        H = np.einsum("eai,eaj->eij", U, dNdx)
        F = np.eye(d) + H
        C = np.einsum("eki,ekj->eij", F, F)
        psi, S, dS, dpsi_dmu, dpsi_dlam = nh_energy_stress(C, mu, lam)
        B = nl_B(F, dNdx)
        Sv = np.stack([S[:, p, q] for p, q in V], axis=1)
        fint += wd[:, None] * np.einsum("evi,ev->ei", B, Sv * m_use)
        fcons += wd[:, None] * np.einsum("evi,ev->ei", B, Sv)
        energy += wd * psi
        Fe += wd[:, None] * (N_matrix(Nv, d).T @ b)[None]
        dmu_de, dlam_de = lame(1.0, nu)
        dEn += (wd * (dpsi_dmu * dmu_de + dpsi_dlam * dlam_de))[:, None] * Nv[None]
        if want_tangent:
            Svm = Sv * m_use
            # geometric part: delta_kl * dN_a^T M dN_b with M built from the used S_voigt
            M = np.zeros((E, d, d), dtype=dt)
            for v, (p, q) in enumerate(V):
                M[:, p, q] = Svm[:, v]
                M[:, q, p] = Svm[:, v]
            G = np.einsum("eap,epq,ebq->eab", dNdx, M, dNdx)
            Kg = np.zeros((E, nd, nd), dtype=dt)
            for k in range(d):
                Kg[:, k::d, k::d] = G
            # material part: B^T (dS_voigt/du)
            Km = np.zeros((E, nd, nd), dtype=dt)
            for bnode in range(nen):
                for l in range(d):
                    dF = np.zeros((E, d, d), dtype=dt)
                    dF[:, l, :] = dNdx[:, bnode, :]
                    dC = np.einsum("eki,ekj->eij", dF, F) + np.einsum("eki,ekj->eij", F, dF)
                    dSt = dS(dC)
                    dSv = np.stack([dSt[:, p, q] for p, q in V], axis=1) * m_use
                    Km[:, :, d * bnode + l] = np.einsum("evi,ev->ei", B, dSv)
            Ke += wd[:, None, None] * (Km + Kg)
    re = fint - Fe
    if squeeze:
        return energy[0], re[0], (Ke[0] if want_tangent else None), fcons[0], dEn[0]
    return energy, re, Ke, fcons, dEn


# --- Neo-Hookean with a volumetric-isochoric split (non-AD variant) ------------
# fol/loss_functions/mechanical_neohooke.py:243-275 with
# fol/constitutive_material_models/neo_hooke.py:14-59 (2-D), 64-111 (3-D).

def bulk_shear(e, nu):
    """kappa, mu from the Young's modulus field at a Gauss point
    (mechanical_neohooke.py:254-255; the same 3-D bulk modulus in 2-D)."""
    return e / (3.0 * (1.0 - 2.0 * nu)), e / (2.0 * (1.0 + nu))


def nh_split_energy_stress(C, kappa, mu):
    """psi = kappa/4 (J^2 - 2 lnJ - 1) + mu/2 (J^(-2/d) I1 - d) in d = 2 or 3
    dimensions (neo_hooke.py:35-38, 87-90) and S = 2 dpsi/dC,
      S = kappa/2 (J^2 - 1) C^-1 + mu J^(-2/d) (I - I1/d C^-1)
    (neo_hooke.py:41-45, 93-97: J p C^-1 + J^(-2/d) P:(mu I)).  Returns psi, S,
    the directional derivative dS(dC) (the reference's C_vol + C_iso,
    neo_hooke.py:47-56, 99-108, is 2 dS/dC), dpsi/dkappa and dpsi/dmu."""
    d = C.shape[-1]
    detC = _det(C)
    lnJ = 0.5 * np.log(detC)
    Ci = _inv(C)
    I1 = np.trace(C, axis1=-2, axis2=-1)
    eye = np.eye(d)
    k_ = kappa[..., None, None]
    mu_ = mu[..., None, None]
    a = np.exp(-2.0 / d * lnJ)                  # J^(-2/d)
    dpsi_dk = 0.25 * (detC - 2.0 * lnJ - 1.0)
    dpsi_dmu = 0.5 * (a * I1 - d)
    psi = kappa * dpsi_dk + mu * dpsi_dmu
    iso = eye - (I1 / d)[..., None, None] * Ci
    S = 0.5 * k_ * (detC - 1.0)[..., None, None] * Ci + mu_ * a[..., None, None] * iso

    def dS(dC):
        trCidC = np.einsum("...ij,...ji->...", Ci, dC)
        dCi = -Ci @ dC @ Ci
        ddet = detC * trCidC
        da = -(1.0 / d) * a * trCidC
        dI1 = np.trace(dC, axis1=-2, axis2=-1)
        diso = -((dI1 / d)[..., None, None] * Ci + (I1 / d)[..., None, None] * dCi)
        return (0.5 * k_ * (ddet[..., None, None] * Ci + (detC - 1.0)[..., None, None] * dCi)
                + mu_ * (da[..., None, None] * iso + a[..., None, None] * diso))

    return psi, S, dS, dpsi_dk, dpsi_dmu


def neohooke_split_element(etype, X, de, ue, num_gp=None, nu=0.3, body_force=None, want_tangent=True):
    """Neo-Hookean element of mechanical_neohooke.py:243-275.

    Per Gauss point kappa, mu from the interpolated Young's modulus
    (:253-255), F = I + H, psi and S of nh_split_energy_stress.  Returns
    (energy, re, Ke, fint, dEnergy/dde) with energy = sum_gp w detJ psi (:266),
    fint = sum_gp w detJ B^T S_voigt (:265, = d energy / d ue), re = fint - Fe
    (:275) and Ke = B^T C_voigt B + the geometric stiffness (:262-263,
    = d re / d ue: the material model's tangent is consistent with its stress).
    """
    X, de, ue, squeeze = _as_batch(X, de, ue)
    nen, d = ELEMENTS[etype]
    if num_gp is None:
        num_gp = 1 if etype == "tet4" else 2
    V = _V3 if d == 3 else _V2
    b = np.zeros(d) if body_force is None else np.asarray(body_force, dtype=np.float64).ravel()[:d]
    pts, wts = gauss_rule(etype, num_gp)
    E = X.shape[0]
    dt = np.result_type(X, de, ue)
    nd = d * nen
    energy = np.zeros(E, dtype=dt)
    fint = np.zeros((E, nd), dtype=dt)
    Fe = np.zeros((E, nd), dtype=dt)
    Ke = np.zeros((E, nd, nd), dtype=dt) if want_tangent else None
    dEn = np.zeros((E, nen), dtype=dt)
    U = ue.reshape(E, nen, d)
    k1, mu1 = bulk_shear(1.0, nu)
    for xi, w in zip(pts, wts):
        Nv = shape_values(etype, xi)
        dNdx, detJ = global_grads(etype, X, xi)
        wd = w * detJ
        kappa, mu = bulk_shear(de @ Nv, nu)
        F = np.eye(d) + np.einsum("eai,eaj->eij", U, dNdx)
        C = np.einsum("eki,ekj->eij", F, F)
        psi, S, dS, dpsi_dk, dpsi_dmu = nh_split_energy_stress(C, kappa, mu)
        B = nl_B(F, dNdx)
        Sv = np.stack([S[:, p, q] for p, q in V], axis=1)
        fint += wd[:, None] * np.einsum("evi,ev->ei", B, Sv)
        energy += wd * psi
        Fe += wd[:, None] * (N_matrix(Nv, d).T @ b)[None]
        dEn += (wd * (k1 * dpsi_dk + mu1 * dpsi_dmu))[:, None] * Nv[None]
        if want_tangent:
            G = np.einsum("eap,epq,ebq->eab", dNdx, S, dNdx)
            Kg = np.zeros((E, nd, nd), dtype=dt)
            for k in range(d):
                Kg[:, k::d, k::d] = G
            Km = np.zeros((E, nd, nd), dtype=dt)
            for bnode in range(nen):
                for l in range(d):
                    dF = np.zeros((E, d, d), dtype=dt)
                    dF[:, l, :] = dNdx[:, bnode, :]
                    dC = np.einsum("eki,ekj->eij", dF, F) + np.einsum("eki,ekj->eij", F, dF)
                    dSt = dS(dC)
                    dSv = np.stack([dSt[:, p, q] for p, q in V], axis=1)
                    Km[:, :, d * bnode + l] = np.einsum("evi,ev->ei", B, dSv)
            Ke += wd[:, None, None] * (Km + Kg)
    re = fint - Fe
    if squeeze:
        return energy[0], re[0], (Ke[0] if want_tangent else None), fint[0], dEn[0]
    return energy, re, Ke, fint, dEn


def transient_thermal_element(etype, X, Tc, Tn, k0, num_gp=2, rho_cp=1.0, dt=1.0, beta=0.0, c=1.0,
                              want_tangent=True):
    """Implicit-Euler transient thermal element (transient_thermal.py:43-78).

    Tc: current nodal temperatures (the control), Tn: next (the unknowns), k0:
    nodal conductivity field.  The element's gradient operator is the
    reference's B = J^-1 dN/dxi^T (transient_thermal.py:57-59), i.e. the
    transpose of J^-1 where ShapeFunctionsGlobalGradients uses J^-T; the two
    agree when J is symmetric, and the golden vectors follow this one.
    Per Gauss point K = (N.k0)(1 + beta T_n^c),
    Se = sum w detJ K dN dN^T, Me = sum w detJ rho cp N N^T.  Returns
    (energy, re, Ke, dEnergy/dTn, dEnergy/dTc) with
      energy = 1/2 Tn.Se(Tn).Tn + sum w detJ rho cp /(2 dt) (T_n - T_c)^2,
      re = (Me + dt Se) Tn - Me Tc,  Ke = Me + dt Se_dR,
      Se_dR = sum w detJ (dK/dT N (x) (grad T . grad N) + K dN dN^T)
    (as written at :64 this is the transpose of d re / d Tn when beta != 0);
    the energy has no stop-gradient, so dEnergy/dTn includes dK/dT."""
    X, Tc, Tn, squeeze = _as_batch(X, Tc, Tn)
    k0 = np.atleast_2d(np.asarray(k0))
    nen, dim = ELEMENTS[etype]
    pts, wts = gauss_rule(etype, num_gp)
    E = X.shape[0]
    dt_ = np.result_type(X, Tc, Tn, k0)
    Se = np.zeros((E, nen, nen), dtype=dt_)
    Me = np.zeros((E, nen, nen), dtype=dt_)
    SdR = np.zeros((E, nen, nen), dtype=dt_)
    tterm = np.zeros(E, dtype=dt_)
    dEn = np.zeros((E, nen), dtype=dt_)
    dEc = np.zeros((E, nen), dtype=dt_)
    for xi, w in zip(pts, wts):
        Nv = shape_values(etype, xi)
        J = jacobian(etype, X, xi)
        detJ = _det(J)
        dNdx = np.einsum("ejk,ak->eaj", _inv(J), shape_local_grads(etype, xi))  # B^T of the reference
        wd = w * detJ
        Tq_n, Tq_c, kq = Tn @ Nv, Tc @ Nv, k0 @ Nv
        K = kq * (1.0 + beta * Tq_n ** c)
        dKdT = kq * beta * c * Tq_n ** (c - 1.0)
        gT = np.einsum("ea,eaj->ej", Tn, dNdx)
        GG = np.einsum("eaj,ebj->eab", dNdx, dNdx)
        Se += (wd * K)[:, None, None] * GG
        Me += (rho_cp * wd)[:, None, None] * np.outer(Nv, Nv)[None]
        diff = Tq_n - Tq_c
        tterm += rho_cp * 0.5 / dt * wd * diff ** 2
        gTN = np.einsum("ej,ebj->eb", gT, dNdx)
        SdR += wd[:, None, None] * (dKdT[:, None, None] * Nv[None, :, None] * gTN[:, None, :]
                                    + K[:, None, None] * GG)
        dEn += wd[:, None] * (K[:, None] * gTN + 0.5 * (dKdT * np.einsum("ej,ej->e", gT, gT))[:, None] * Nv[None]
                              + (rho_cp / dt * diff)[:, None] * Nv[None])
        dEc -= (wd * rho_cp / dt * diff)[:, None] * Nv[None]
    energy = 0.5 * np.einsum("ea,eab,eb->e", Tn, Se, Tn) + tterm
    re = np.einsum("eab,eb->ea", Me + dt * Se, Tn) - np.einsum("eab,eb->ea", Me, Tc)
    Ke = Me + dt * SdR
    if squeeze:
        return energy[0], re[0], Ke[0], dEn[0], dEc[0]
    return energy, re, Ke, dEn, dEc


def saint_venant_element(etype, X, de, ue, num_gp=None, nu=0.3, body_force=None, want_tangent=True):
    """Saint-Venant-Kirchhoff element (mechanical_saint_venant.py:263-296 with
    constitutive_material_models/saint_venant.py:13-31).

    Per Gauss point: lam, mu from the interpolated Young's modulus (3-D Lame
    constants, also in 2-D, :274-276), F = I + H, E = (F^T F - I)/2,
    psi = lam/2 tr(E)^2 + mu E:E, S = lam tr(E) I + 2 mu E.  Returns
    (energy, re, Ke, fint, dEnergy/dde) with energy = sum_gp w detJ psi,
    fint = sum_gp w detJ B^T S_voigt (= d energy / d ue), re = fint - Fe and
    Ke = B^T C B + the geometric stiffness (d re / d ue)."""
    X, de, ue, squeeze = _as_batch(X, de, ue)
    nen, d = ELEMENTS[etype]
    if num_gp is None:
        num_gp = 1 if etype == "tet4" else 2
    V = _V3 if d == 3 else _V2
    b = np.zeros(d) if body_force is None else np.asarray(body_force, dtype=np.float64).ravel()[:d]
    pts, wts = gauss_rule(etype, num_gp)
    E = X.shape[0]
    dt = np.result_type(X, de, ue)
    nd = d * nen
    energy = np.zeros(E, dtype=dt)
    fint = np.zeros((E, nd), dtype=dt)
    Fe = np.zeros((E, nd), dtype=dt)
    Ke = np.zeros((E, nd, nd), dtype=dt) if want_tangent else None
    dEn = np.zeros((E, nen), dtype=dt)
    U = ue.reshape(E, nen, d)
    eye = np.eye(d)
    for xi, w in zip(pts, wts):
        Nv = shape_values(etype, xi)
        dNdx, detJ = global_grads(etype, X, xi)
        wd = w * detJ
        egp = de @ Nv
        mu, lam = lame(egp, nu)
        mu1, lam1 = lame(1.0, nu)
        H = np.einsum("eai,eaj->eij", U, dNdx)
        F = eye + H
        Es = 0.5 * (np.einsum("eki,ekj->eij", F, F) - eye)
        trE = np.einsum("eii->e", Es)
        EE = np.einsum("eij,eij->e", Es, Es)
        psi = 0.5 * lam * trE ** 2 + mu * EE
        S = lam[:, None, None] * trE[:, None, None] * eye + 2.0 * mu[:, None, None] * Es
        B = nl_B(F, dNdx)
        Sv = np.stack([S[:, p, q] for p, q in V], axis=1)
        fint += wd[:, None] * np.einsum("evi,ev->ei", B, Sv)
        energy += wd * psi
        Fe += wd[:, None] * (N_matrix(Nv, d).T @ b)[None]
        dEn += (wd * (0.5 * lam1 * trE ** 2 + mu1 * EE))[:, None] * Nv[None]
        if want_tangent:
            G = np.einsum("eap,epq,ebq->eab", dNdx, S, dNdx)
            Kg = np.zeros((E, nd, nd), dtype=dt)
            for k in range(d):
                Kg[:, k::d, k::d] = G
            Km = np.zeros((E, nd, nd), dtype=dt)
            for bnode in range(nen):
                for l in range(d):
                    dF = np.zeros((E, d, d), dtype=dt)
                    dF[:, l, :] = dNdx[:, bnode, :]
                    dE = 0.5 * (np.einsum("eki,ekj->eij", dF, F) + np.einsum("eki,ekj->eij", F, dF))
                    dS = (lam[:, None, None] * np.einsum("eii->e", dE)[:, None, None] * eye
                          + 2.0 * mu[:, None, None] * dE)
                    dSv = np.stack([dS[:, p, q] for p, q in V], axis=1)
                    Km[:, :, d * bnode + l] = np.einsum("evi,ev->ei", B, dSv)
            Ke += wd[:, None, None] * (Km + Kg)
    re = fint - Fe
    if squeeze:
        return energy[0], re[0], (Ke[0] if want_tangent else None), fint[0], dEn[0]
    return energy, re, Ke, fint, dEn


# ----------------------------------------------------------------------------
# Mesh generators (structured, seeded) — node/element ordering of the reference
# ----------------------------------------------------------------------------

def square_mesh(L, N):
    """create_2D_square_mesh (fol/tools/usefull_functions.py:213-258):
    x-fastest node numbering, quad4 elements, 'left'/'right' node sets."""
    Ne = N - 1
    x = np.linspace(0, L, N)
    X, Y = np.meshgrid(x, x)
    xyz = np.stack([X.ravel(), Y.ravel(), np.zeros(N * N)], axis=1)
    i, j = np.meshgrid(np.arange(Ne), np.arange(Ne), indexing="ij")
    i, j = i.ravel(), j.ravel()
    conn = np.stack([i * N + j, i * N + j + 1, (i + 1) * N + j + 1, (i + 1) * N + j], axis=1)
    sets = {"left": np.arange(0, N * N, N), "right": np.arange(N - 1, N * N, N)}
    return xyz, conn.astype(np.int64), sets


# ----------------------------------------------------------------------------
# FE loss: DOF bookkeeping, gather, loss, residual, Jacobian
#   fol/loss_functions/fe_loss.py
# ----------------------------------------------------------------------------

PHYSICS_NDOF = {"thermal": lambda dim: 1, "elastic": lambda dim: dim, "neohooke": lambda dim: dim,
                "saint_venant": lambda dim: dim, "transient_thermal": lambda dim: 1,
                "neohooke_split": lambda dim: dim}


class FELossOracle:
    """Restatement of FiniteElementLoss (fe_loss.py:19-318) for one element type.

    physics: "thermal" (thermal.py), "elastic" (mechanical.py) or "neohooke"
    (mechanical_neohooke_AD.py).  control_layout "nodal" gathers the control
    by connectivity as the reference does (fe_loss.py:160); "element" takes one
    value per element and uses de = value * 1 (partition of unity).
    """

    def __init__(self, etype, physics, xyz, conn, dirichlet=None, node_sets=None,
                 num_gp=None, young=1.0, nu=0.3, body_force=None, beta=0.0, c=1.0,
                 exponent=1.0, shear_mode="reference", control_layout="nodal",
                 rho_cp=1.0, time_step=1.0, material_beta=0.0, k0=None):
        self.etype, self.physics = etype, physics
        self.nen, self.dim = ELEMENTS[etype]
        self.ndof = PHYSICS_NDOF[physics](self.dim)
        self.xyz = np.asarray(xyz, dtype=np.float64)
        self.conn = np.asarray(conn, dtype=np.int64)
        self.num_nodes = len(self.xyz)
        self.num_gp = num_gp if num_gp is not None else (1 if etype == "tet4" else 2)
        self.young, self.nu, self.beta, self.c = young, nu, beta, c
        self.body_force = body_force
        self.exponent = exponent
        self.shear_mode = shear_mode
        self.control_layout = control_layout
        # transient thermal (transient_thermal.py:20-41): the control is the
        # current temperature field, k0 a nodal conductivity field
        self.rho_cp, self.time_step, self.material_beta = rho_cp, time_step, material_beta
        self.k0 = np.ones(len(xyz)) if k0 is None else np.asarray(k0, dtype=np.float64)
        self.total_dofs = self.ndof * self.num_nodes
        # __CreateDofsDict (fe_loss.py:34-55)
        idx, val = [], []
        dofnames = ["T"] if self.ndof == 1 else ["Ux", "Uy", "Uz"][: self.ndof]
        dirichlet = dirichlet or {}
        for di, name in enumerate(dofnames):
            for set_name, value in dirichlet.get(name, {}).items():
                nodes = np.asarray(node_sets[set_name], dtype=np.int64)
                idx.append(self.ndof * nodes + di)
                val.append(np.full(len(nodes), float(value)))
        self.dirichlet_indices = np.concatenate(idx) if idx else np.zeros(0, np.int64)
        self.dirichlet_values = np.concatenate(val) if val else np.zeros(0)
        self.non_dirichlet_indices = np.setdiff1d(np.arange(self.total_dofs), self.dirichlet_indices)

    # ---- fe_loss.py:91-100, 186-189
    def full_dof_vector(self, u, load_increment=1.0):
        u = np.array(u, dtype=np.result_type(u, np.float64), copy=True)
        u[..., self.dirichlet_indices] = load_increment * self.dirichlet_values
        return u

    def _gather(self, ctrl, u):
        X = self.xyz[self.conn]
        if self.control_layout == "element":
            de = np.repeat(np.asarray(ctrl)[:, None], self.nen, axis=1)
        else:
            de = np.asarray(ctrl)[self.conn]
        dofidx = (self.ndof * self.conn[:, :, None] + np.arange(self.ndof)).reshape(len(self.conn), -1)
        return X, de, np.asarray(u)[dofidx], dofidx

    def element(self, X, de, ue, want_tangent=True):
        """Returns (energy, re, Ke, energy_grad_u, energy_grad_de) per element."""
        if self.physics == "thermal":
            en, re, Ke, dEn = thermal_element(self.etype, X, de, ue, self.num_gp, self.beta, self.c)
            return en, re, Ke, re, dEn
        if self.physics == "elastic":
            en, re, Ke, dEn = linear_elastic_element(self.etype, X, de, ue, self.num_gp,
                                                     self.young, self.nu, self.body_force)
            return en, re, Ke, re, dEn
        if self.physics == "saint_venant":
            return saint_venant_element(self.etype, X, de, ue, self.num_gp, self.nu, self.body_force, want_tangent)
        if self.physics == "neohooke_split":
            return neohooke_split_element(self.etype, X, de, ue, self.num_gp, self.nu, self.body_force, want_tangent)
        if self.physics == "transient_thermal":
            en, re, Ke, dEn, dEc = transient_thermal_element(self.etype, X, de, ue, self.k0[self.conn], self.num_gp,
                                                             self.rho_cp, self.time_step, self.material_beta, self.c)
            return en, re, Ke, dEn, dEc
        en, re, Ke, fcons, dEn = neohooke_element(self.etype, X, de, ue, self.num_gp, self.nu,
                                                  self.body_force, self.shear_mode, want_tangent)
        return en, re, Ke, fcons, dEn

    # ---- fe_loss.py:166-176
    def element_energies(self, ctrl, u):
        X, de, ue, _ = self._gather(ctrl, u)
        return self.element(X, de, ue, want_tangent=False)[0]

    def total_energy(self, ctrl, u):
        return float(np.sum(self.element_energies(ctrl, u)))

    def _assemble_nodal(self, vals_e, ncomp):
        out = np.zeros(ncomp * self.num_nodes, dtype=vals_e.dtype)
        idx = (ncomp * self.conn[:, :, None] + np.arange(ncomp)).reshape(len(self.conn), -1)
        np.add.at(out, idx.ravel(), vals_e.reshape(len(self.conn), -1).ravel())
        return out

    # ---- fe_loss.py:250-262 plus its adjoint (what jax.grad of the batch loss gives
    #      for u; the FD-of-value derivative for the control)
    def batch_loss_and_grads(self, batch_ctrl, batch_u):
        """Returns (mean, (min, max, mean), per-instance losses, dLoss/du, dLoss/dctrl).

        batch_u holds full DOF vectors; Dirichlet entries are overwritten first
        (GetFullDofVector), so their gradient is zero.
        """
        batch_ctrl = np.atleast_2d(np.asarray(batch_ctrl, dtype=np.float64))
        batch_u = np.atleast_2d(np.asarray(batch_u, dtype=np.float64))
        B = batch_u.shape[0]
        if batch_ctrl.shape[0] == 1 and B > 1:
            batch_ctrl = np.repeat(batch_ctrl, B, axis=0)
        p = self.exponent
        losses = np.zeros(B)
        du = np.zeros_like(batch_u)
        dctrl = np.zeros_like(batch_ctrl)
        for b in range(B):
            u = self.full_dof_vector(batch_u[b])
            X, de, ue, _ = self._gather(batch_ctrl[b], u)
            en, re, _, gu, gde = self.element(X, de, ue, want_tangent=False)
            tot = float(np.sum(en))
            losses[b] = tot ** p
            scale = p * tot ** (p - 1.0) / B if p != 1.0 else 1.0 / B
            g = self._assemble_nodal(gu, self.ndof)
            g[self.dirichlet_indices] = 0.0
            du[b] = scale * g
            if self.control_layout == "element":
                dctrl[b] = scale * gde.sum(axis=1)
            else:
                dctrl[b] = scale * self._assemble_nodal(gde, 1)
        return losses.mean(), (losses.min(), losses.max(), losses.mean()), losses, du, dctrl

    # ---- fe_loss.py:191-207 (row-only Dirichlet on the element system)
    def _bc_vectors(self):
        bc = np.ones(self.total_dofs)
        bc[self.dirichlet_indices] = 0.0
        mask = np.zeros(self.total_dofs)
        mask[self.dirichlet_indices] = 1.0
        return bc, mask

    def element_residuals_and_jacobians(self, ctrl, u, transpose=False):
        """BC-applied element residuals (E, nd) and matrices (E, nd, nd)
        (fe_loss.py:209-248)."""
        X, de, ue, dofidx = self._gather(ctrl, u)
        _, re, Ke, _, _ = self.element(X, de, ue, want_tangent=True)
        if transpose:
            Ke = np.swapaxes(Ke, 1, 2)
        bc, mask = self._bc_vectors()
        bce, mke = bc[dofidx], mask[dofidx]
        diag = np.einsum("eii->ei", Ke) * mke
        Kbc = bce[:, :, None] * Ke
        idx = np.arange(Ke.shape[1])
        Kbc[:, idx, idx] += diag
        return bce * re, Kbc, dofidx

    def residual_and_jacobian(self, ctrl, u, transpose=False):
        """ComputeJacobianMatrixAndResidualVector (fe_loss.py:264-318): assembled
        residual and the duplicate-laden COO (rows, cols, values)."""
        re, Ke, dofidx = self.element_residuals_and_jacobians(ctrl, u, transpose)
        R = np.zeros(self.total_dofs)
        np.add.at(R, dofidx.ravel(), re.ravel())
        nd = dofidx.shape[1]
        rows = np.repeat(dofidx, nd, axis=1).ravel()
        cols = np.tile(dofidx, (1, nd)).ravel()
        return R, (rows, cols, Ke.ravel())

    def csr(self, ctrl, u, transpose=False):
        """Canonical CSR of the BC-applied Jacobian, built exactly the way the
        reference converts its BCOO (fe_solver.py:71-72)."""
        R, (rows, cols, vals) = self.residual_and_jacobian(ctrl, u, transpose)
        A = sp.csr_array((vals, (rows, cols)), shape=(self.total_dofs, self.total_dofs))
        A.sum_duplicates()
        A.sort_indices()
        return A, R


# ----------------------------------------------------------------------------
# Nodal Fourier control (fol/controls/fourier_control.py:24-59)
# ----------------------------------------------------------------------------

def fourier_frequencies(x_freqs, y_freqs, z_freqs):
    """meshgrid(x, y, z, indexing="ij") flattened row-major (fourier_control.py:44-45)."""
    mx, my, mz = np.meshgrid(np.asarray(x_freqs, float), np.asarray(y_freqs, float), np.asarray(z_freqs, float),
                             indexing="ij")
    return np.stack([mx.ravel(), my.ravel(), mz.ravel()], axis=1)


def fourier_basis(freqs, xyz):
    """(F, N): cos(fx pi x) cos(fy pi y) cos(fz pi z) per frequency and node (:53-57)."""
    X = np.asarray(xyz, dtype=np.float64)
    return (np.cos(np.pi * freqs[:, 0:1] * X[None, :, 0]) * np.cos(np.pi * freqs[:, 1:2] * X[None, :, 1])
            * np.cos(np.pi * freqs[:, 2:3] * X[None, :, 2]))


def fourier_control_values(coeffs, freqs, xyz, vmin=1e-6, vmax=1.0, beta=1.0, scale_min=0.0, scale_max=1.0):
    """ComputeControlledVariables (:49-59): coeffs (B, F+1) -> nodal values (B, N)."""
    v = np.atleast_2d(np.asarray(coeffs, dtype=np.float64)) * (scale_max - scale_min) + scale_min
    K = v[:, :1] / 2.0 + v[:, 1:] @ fourier_basis(freqs, xyz)
    return (vmax - vmin) / (1.0 + np.exp(-beta * (K - 0.5))) + vmin


def fourier_control_vjp(coeffs, dvalues, freqs, xyz, vmin=1e-6, vmax=1.0, beta=1.0, scale_min=0.0,
                        scale_max=1.0):
    """d(sum dvalues * values)/d coeffs (B, F+1): what jax.grad through the
    control gives for a loss whose nodal-control gradient is dvalues."""
    v = np.atleast_2d(np.asarray(coeffs, dtype=np.float64)) * (scale_max - scale_min) + scale_min
    Phi = fourier_basis(freqs, xyz)
    K = v[:, :1] / 2.0 + v[:, 1:] @ Phi
    s = 1.0 / (1.0 + np.exp(-beta * (K - 0.5)))
    g = np.atleast_2d(dvalues) * (vmax - vmin) * beta * s * (1.0 - s)
    return (scale_max - scale_min) * np.concatenate([0.5 * g.sum(axis=1, keepdims=True), g @ Phi.T], axis=1)


# ----------------------------------------------------------------------------
# Solvers
# ----------------------------------------------------------------------------

def direct_solve(A, b):
    """FP64 direct solve (the JAX-direct path of fe_solver.py:70-78)."""
    return spla.spsolve(sp.csc_matrix(A), b)


def jacobi_pcg(A, b, rtol=1e-8, maxiter=10000):
    """Jacobi-preconditioned CG with x0 = 0 in FP64 (the GPU solver's algorithm).
    Returns (x, iterations, final relative residual)."""
    A = sp.csr_array(A)
    dinv = 1.0 / A.diagonal()
    x = np.zeros_like(b)
    r = b.copy()
    z = dinv * r
    p = z.copy()
    rz = r @ z
    bn = np.linalg.norm(b)
    if bn == 0.0:
        return x, 0, 0.0
    for it in range(1, maxiter + 1):
        Ap = A @ p
        alpha = rz / (p @ Ap)
        x += alpha * p
        r -= alpha * Ap
        rn = np.linalg.norm(r)
        if rn <= rtol * bn:
            return x, it, rn / bn
        z = dinv * r
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
    return x, maxiter, np.linalg.norm(r) / bn


def linear_solve(loss: FELossOracle, ctrl, u0):
    """FiniteElementLinearResidualBasedSolver.Solve (fe_linear_residual_based_solver.py:15-22)
    with the direct solver."""
    u = loss.full_dof_vector(u0)
    A, R = loss.csr(ctrl, u)
    return u + direct_solve(A, -R)


def newton_solve(loss: FELossOracle, ctrl, u0, load_incr=5, maxiter=20, abs_tol=1e-8, rel_tol=1e-8,
                 line_search=False, max_halvings=30):
    """FiniteElementNonLinearResidualBasedSolver.Solve
    (fe_nonlinear_residual_based_solver.py:76-170): load stepping, Newton,
    convergence on |r| < abs_tol or |du| < rel_tol or maxiter; the converged
    step's update is not applied (:162-166).  line_search=True (not in the
    reference, which takes full steps): backtracking on the total energy,
    t = 1, 1/2, ... until E(u + t du) <= E(u) - 1e-4 t max(-(r . du), 0) and
    finite, with du replaced by the Jacobi-preconditioned steepest descent
    step -D^-1 r when the Newton step is not a descent direction (FP64; for
    losses whose residual is the energy gradient)."""
    u = np.array(u0, dtype=np.float64, copy=True)
    history = []
    for step in range(1, load_incr + 1):
        u = loss.full_dof_vector(u, step / load_incr)
        for it in range(1, maxiter + 1):
            A, R = loss.csr(ctrl, u)
            rn = np.linalg.norm(R)
            if not np.isfinite(rn):
                raise ValueError("Residual norm contains NaN values.")
            du = direct_solve(A, -R)
            dn = np.linalg.norm(du)
            history.append((step, it, rn, dn))
            if rn < abs_tol or dn < rel_tol or it == maxiter:
                break
            t = 1.0
            if line_search:
                with np.errstate(all="ignore"):
                    e0 = loss.total_energy(ctrl, u)
                    slope = -float(R @ du)
                    if not np.isfinite(dn) or slope <= 0.0:
                        # not a descent direction (indefinite tangent): the
                        # Jacobi-preconditioned steepest descent step instead
                        du = -R / A.diagonal()
                        slope = -float(R @ du)
                    for _ in range(max_halvings + 1):
                        et = loss.total_energy(ctrl, u + t * du)
                        if np.isfinite(et) and et <= e0 - 1e-4 * t * max(slope, 0.0):
                            break
                        t *= 0.5
                    else:
                        raise ValueError("line search found no decrease")
            u = u + t * du
    return u, history


# ----------------------------------------------------------------------------
# Adjoint sensitivities of a response  (fol/responses/fe_response.py)
# ----------------------------------------------------------------------------

def _complex_step(fun, x, h=1e-30):
    """d fun / d x for every entry of x by the complex-step method
    (Squire & Trapp 1998): exact to rounding for analytic fun."""
    x = np.asarray(x, dtype=np.complex128)
    cols = []
    for i in range(x.size):
        xp = x.copy().ravel()
        xp[i] += 1j * h
        cols.append(np.imag(fun(xp.reshape(x.shape))) / h)
    return np.stack(cols, axis=-1)


class ResponseOracle:
    """Integral response J = sum_e sum_gp w detJ f(d_gp, u_gp) over a thermal or
    elastic loss (fe_response.py:92-120), f = sum_k c_k d^p_k prod_i u_i^q_ki
    given as monomials [(c, p, (q_0, q_1, q_2)), ...], and its adjoint
    sensitivities (fe_response.py:244-526) by complex-step differentiation of
    the element value and the element residual."""

    def __init__(self, loss: FELossOracle, monomials):
        assert loss.physics in ("thermal", "elastic")
        self.loss = loss
        self.monomials = [(float(c), int(p), tuple(int(v) for v in q)) for c, p, q in monomials]

    def f(self, d, u):
        out = 0.0
        for c, p, q in self.monomials:
            term = c * d ** p
            for i in range(len(u)):
                term = term * u[i] ** q[i]
            out = out + term
        return out

    def element_value(self, X, de, ue):
        L = self.loss
        pts, wts = gauss_rule(L.etype, L.num_gp)
        val = 0.0
        for xi, w in zip(pts, wts):
            Nv = shape_values(L.etype, xi)
            detJ = _det(jacobian(L.etype, X, xi))
            uq = N_matrix(Nv, L.ndof) @ ue
            val = val + w * detJ * self.f(Nv @ de, uq)
        return val

    def _de(self, ctrl, e, nodes):
        if self.loss.control_layout == "element":
            return np.full(len(nodes), np.asarray(ctrl)[e], dtype=np.result_type(np.asarray(ctrl), float))
        return np.asarray(ctrl)[nodes]

    def _per_element(self, fn, ctrl, u, adj=None):
        L = self.loss
        out = []
        for e in range(len(L.conn)):
            nodes = L.conn[e]
            X = L.xyz[nodes]
            dofs = (L.ndof * nodes[:, None] + np.arange(L.ndof)).ravel()
            ue = np.asarray(u)[dofs]
            ae = None if adj is None else np.asarray(adj)[dofs]
            out.append(fn(X, self._de(ctrl, e, nodes), ue, ae))
        return np.array(out)

    def value(self, ctrl, u):
        """ComputeValue (fe_response.py:208-225)."""
        return float(np.sum(self._per_element(lambda X, de, ue, _: self.element_value(X, de, ue), ctrl, u)))

    def adjoint_jacobian_and_rhs(self, ctrl, u):
        """ComputeAdjointJacobianMatrixAndRHSVector (fe_response.py:244-283)."""
        L = self.loss
        g = self._per_element(lambda X, de, ue, _: _complex_step(lambda v: self.element_value(X, de, v), ue), ctrl, u)
        rhs = L._assemble_nodal(g, L.ndof)
        rhs[L.dirichlet_indices] = 0.0
        rhs *= -1.0
        A, _ = L.csr(ctrl, u, transpose=True)
        return A, rhs

    def _residual(self, X, de, ue):
        L = self.loss
        if L.physics == "thermal":
            return thermal_element(L.etype, X, de, ue, L.num_gp, L.beta, L.c)[1]
        return linear_elastic_element(L.etype, X, de, ue, L.num_gp, L.young, L.nu, L.body_force)[1]

    def nodal_control_derivatives(self, ctrl, u, adj):
        """ComputeAdjointNodalControlDerivatives (fe_response.py:486-526); for
        element controls the per-element sums."""
        L = self.loss

        def per(X, de, ue, ae):
            dR = _complex_step(lambda d: self.element_value(X, d, ue), de)
            dres = _complex_step(lambda d: self._residual(X, d, ue), de)   # (nd, nen)
            return dR + ae @ dres
        g = self._per_element(per, ctrl, u, adj)
        if L.control_layout == "element":
            return g.sum(axis=1)
        return L._assemble_nodal(g, 1)

    def nodal_shape_derivatives(self, ctrl, u, adj):
        """ComputeAdjointNodalShapeDerivatives (fe_response.py:365-406)."""
        L = self.loss

        def per(X, de, ue, ae):
            dR = _complex_step(lambda x: self.element_value(x, de, ue), X)
            dres = _complex_step(lambda x: self._residual(x, de, ue), X)   # (nd, nen*3)
            return dR + ae @ dres
        return L._assemble_nodal(self._per_element(per, ctrl, u, adj), 3)


class QuadResponseOracle(ResponseOracle):
    """The "(E**2)*U[0]" response on a quad4 elastic loss
    (tests/unit/test_sensitivity_analysis.py:477)."""

    def __init__(self, loss: FELossOracle):
        assert loss.etype == "quad4" and loss.physics == "elastic"
        super().__init__(loss, [(1.0, 2, (1, 0, 0))])
