"""Full-size parity: the CUDA path against the C FP64 oracle at the sizes the
benchmark runs (64^3 hex8 elasticity with a two-phase voxel field, element
controls) and at large generic-kernel sizes.  Tolerance 1e-5 relative
(Frobenius) on the losses and both gradients."""
import numpy as np
import pytest

from gpu_cases import c_oracle_loss, gpu_loss, make_mesh, rel_fro
from folax_gb300 import fields
from folax_gb300.mesh import create_3D_box_mesh

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _compare(gl, cl, ctrl, u):
    a = gl.ComputeBatchLossAndGrad(ctrl, u)
    o = cl.batch_loss_and_grads(ctrl, u)
    gl.CheckDeviceStatus()
    for x, z in zip(a[2:], o[2:]):
        assert rel_fro(x.cpu().numpy(), z) < TOL


@pytest.mark.parametrize("variant", ["auto", 0, 2, 15, 18, 19, 20, 21, 22, 23, 24])
def test_hex8_64_cubed_two_phase_matches_c_oracle(cuda, variant):
    n = 64
    m = create_3D_box_mesh(n, n, n)
    s = {"dirichlet_bc_dict": {"Ux": {"bottom": 0.0}, "Uy": {"bottom": 0.0}, "Uz": {"bottom": 0.0, "top": 0.05}},
         "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3}, "control_layout": "element"}
    gl = gpu_loss("hex8", "elastic", m, {**s, "kernel_variant": variant})
    cl = c_oracle_loss("hex8", "elastic", m, s)
    E = fields.two_phase_voxels(n, 2024, sigma=3.0, high=1.0, low=0.1)[None]
    rng = np.random.default_rng(2025)
    u = np.zeros((m.GetNumberOfNodes(), 3))
    u[:, 2] = 0.05 * m.nodes_coordinates[:, 2]
    u = (u + 0.01 * rng.standard_normal(u.shape)).reshape(1, -1)
    if variant == "auto":
        gl.Autotune(E, u, repeats=2)
    _compare(gl, cl, E, u)


@pytest.mark.parametrize("etype,physics,n", [("hex8", "thermal", 40), ("tet4", "elastic", 24), ("quad4", "elastic", 256),
                                             ("tet4", "thermal", 24), ("quad4", "thermal", 256)])
@pytest.mark.parametrize("layout", ["nodal", "element"])
def test_large_generic_cases_match_c_oracle(cuda, etype, physics, n, layout):
    m = make_mesh(etype, n, seed=31)
    from gpu_cases import bc_dict
    s = {"dirichlet_bc_dict": bc_dict(etype, physics), "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3},
         "control_layout": layout}
    gl, cl = gpu_loss(etype, physics, m, s), c_oracle_loss(etype, physics, m, s)
    rng = np.random.default_rng(32)
    ctrl = 0.5 + rng.random((2, gl.GetNumberOfControls()))
    u = (0.05 / n) * rng.standard_normal((2, gl.GetTotalNumberOfDOFs()))
    _compare(gl, cl, ctrl, u)


# Batches big enough that each block of the generic element kernel takes
# several element ranges: tet4 24^3 split (82,944 tets, 324 ranges of 256) at
# batch 32 gives 2 ranges per block; quad4 256^2 (256 ranges) at batch 80,
# 160 and 320 gives 4, 8 and 16, on a 152-SM GPU (at least 8 waves of 4
# blocks per SM each time).
@pytest.mark.parametrize("etype,physics,n,batch", [("tet4", "elastic", 24, 32), ("quad4", "thermal", 256, 80),
                                                   ("quad4", "thermal", 256, 160), ("quad4", "elastic", 256, 320)])
def test_multi_range_blocks_match_c_oracle(cuda, etype, physics, n, batch):
    m = make_mesh(etype, n, seed=33)
    from gpu_cases import bc_dict
    s = {"dirichlet_bc_dict": bc_dict(etype, physics), "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3},
         "control_layout": "element"}
    gl, cl = gpu_loss(etype, physics, m, s), c_oracle_loss(etype, physics, m, s)
    rng = np.random.default_rng(34)
    ctrl = 0.5 + rng.random((batch, gl.GetNumberOfControls()))
    u = (0.05 / n) * rng.standard_normal((batch, gl.GetTotalNumberOfDOFs()))
    _compare(gl, cl, ctrl, u)
