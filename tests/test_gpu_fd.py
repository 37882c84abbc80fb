"""Differentiation check at 32^3 (hex8 elasticity, two-phase voxel field,
element controls): the GPU adjoint against FP64 central differences (h = 1e-4)
of the C oracle's loss along 64 seeded random directions in u and 64 in E.

The loss is L = u . stop_gradient(K(E) u - f) (mechanical.py:114-117), so
  * dL/du returned by the adjoint is the residual K u - f, the gradient of the
    potential 1/2 u.K u - u.f: its directional derivative is FD(L)/2 for f = 0;
  * dL/dE is the derivative of the loss value: FD(L) along e.
Per direction: |g.d - FD| <= 1e-5 |g| |d|."""
import numpy as np
import pytest

from gpu_cases import c_oracle_loss, gpu_loss
from folax_gb300 import fields
from folax_gb300.mesh import create_3D_box_mesh

pytestmark = pytest.mark.gpu
TOL = 1e-5
H = 1e-4
DIRECTIONS = 64


def test_adjoint_matches_fp64_central_differences_32cubed(cuda):
    n = 32
    m = create_3D_box_mesh(n, n, n)
    s = {"dirichlet_bc_dict": {"Ux": {"bottom": 0.0}, "Uy": {"bottom": 0.0}, "Uz": {"bottom": 0.0, "top": 0.05}},
         "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3}, "control_layout": "element"}
    gl = gpu_loss("hex8", "elastic", m, s)
    cl = c_oracle_loss("hex8", "elastic", m, s)
    E = fields.two_phase_voxels(n, 2024, sigma=3.0, high=1.0, low=0.1).astype(np.float64)
    rng = np.random.default_rng(2026)
    u = np.zeros((m.GetNumberOfNodes(), 3))
    u[:, 2] = 0.05 * m.nodes_coordinates[:, 2]
    u = cl.py.full_dof_vector(u.ravel() + 0.01 * rng.standard_normal(3 * m.GetNumberOfNodes()))
    _, _, _, du, dE = gl.ComputeBatchLossAndGrad(E[None], u[None])
    gl.CheckDeviceStatus()
    du = du[0].double().cpu().numpy()
    dE = dE[0].double().cpu().numpy()
    free = cl.py.non_dirichlet_indices

    def loss(Ev, uv):
        return cl.loss_adjoint(Ev, uv)[0]

    worst_u = worst_e = 0.0
    for _ in range(DIRECTIONS):
        d = np.zeros_like(u)
        d[free] = rng.standard_normal(len(free))
        fd = (loss(E, u + H * d) - loss(E, u - H * d)) / (2 * H)
        err = abs(du @ d - 0.5 * fd) / (np.linalg.norm(du) * np.linalg.norm(d))
        worst_u = max(worst_u, err)
        e = rng.standard_normal(len(E))
        fd = (loss(E + H * e, u) - loss(E - H * e, u)) / (2 * H)
        err = abs(dE @ e - fd) / (np.linalg.norm(dE) * np.linalg.norm(e))
        worst_e = max(worst_e, err)
    assert worst_u < TOL, worst_u
    assert worst_e < TOL, worst_e
