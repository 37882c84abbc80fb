"""Nodal Fourier control on the GPU (fourier_control.py:14-59) against the FP64
oracle, alone and chained in front of the fused loss + adjoint (the FOL
training step), eagerly and as one CUDA graph.  Tolerance 1e-5 relative."""
import numpy as np
import pytest

from gpu_cases import bc_dict, gpu_loss, make_mesh, oracle_loss, rel_fro
from oracle import fe_oracle as fo

pytestmark = pytest.mark.gpu
TOL = 1e-5

SETTINGS = {"x_freqs": np.array([1, 2, 3]), "y_freqs": np.array([0, 2]), "z_freqs": np.array([1, 4]),
            "beta": 4.0, "min": 0.1, "max": 1.0}


def _control(mesh, settings=SETTINGS, scale=(0.0, 1.0)):
    from folax_gb300.fields import FourierControl
    fc = FourierControl("E", settings, mesh)
    fc.scale_min, fc.scale_max = scale
    fc.Initialize()
    return fc


def _oracle_kw(settings=SETTINGS, scale=(0.0, 1.0)):
    return dict(vmin=settings["min"], vmax=settings["max"], beta=settings["beta"], scale_min=scale[0],
                scale_max=scale[1])


def _xyz(mesh):
    X = np.zeros((mesh.GetNumberOfNodes(), 3))
    X[:, : mesh.nodes_coordinates.shape[1]] = mesh.nodes_coordinates
    return X


# more than four frequencies on an axis: several 4 x 4 x 4 tiles of the
# frequency grid, with partly empty edge tiles
WIDE = {"x_freqs": np.arange(0, 6), "y_freqs": np.array([1, 3]), "z_freqs": np.array([0, 1, 2, 3, 5]),
        "beta": 4.0, "min": 0.1, "max": 1.0}
# more than 64 tiles: the forward kernels read the coefficients in plain order
MANY = {"x_freqs": np.arange(0, 17), "y_freqs": np.arange(0, 17), "z_freqs": np.arange(0, 13),
        "beta": 4.0, "min": 0.1, "max": 1.0}


@pytest.mark.parametrize("etype,n,scale,settings", [("hex8", 12, (0.0, 1.0), SETTINGS),
                                                    ("quad4", 40, (-0.5, 1.5), SETTINGS),
                                                    ("tet4", 6, (0.0, 1.0), SETTINGS),
                                                    ("hex8", 12, (0.0, 1.0), WIDE),
                                                    ("quad4", 40, (-0.5, 1.5), WIDE),
                                                    ("hex8", 8, (0.0, 1.0), MANY)])
def test_fourier_forward_and_vjp_match_oracle(cuda, etype, n, scale, settings):
    torch = cuda
    m = make_mesh(etype, n, seed=41)
    fc = _control(m, settings=settings, scale=scale)
    freqs = fo.fourier_frequencies(settings["x_freqs"], settings["y_freqs"], settings["z_freqs"])
    rng = np.random.default_rng(42)
    F = fc.GetNumberOfVariables()
    # K's spread kept near one for big bases, so the sigmoid is not saturated
    c = 0.5 * min(1.0, np.sqrt(64 / F)) * rng.standard_normal((3, F))
    vals = fc.ComputeBatchControlledVariables(c)
    ref = fo.fourier_control_values(c, freqs, _xyz(m), **_oracle_kw(settings, scale=scale))
    assert rel_fro(vals.cpu().numpy(), ref) < TOL
    assert rel_fro(fc.ComputeControlledVariables(c[1]).cpu().numpy(), ref[1]) < TOL
    dv = rng.standard_normal((3, fc.GetNumberOfControlledVariables()))
    g = fc.ComputeBatchControlledVariablesVJP(c, dv)
    gref = fo.fourier_control_vjp(c, dv, freqs, _xyz(m), **_oracle_kw(settings, scale=scale))
    assert rel_fro(g.cpu().numpy(), gref) < TOL
    # deterministic: the same launch twice gives the same bits
    assert torch.equal(g, fc.ComputeBatchControlledVariablesVJP(c, dv))


def test_fourier_control_in_front_of_fused_loss(cuda):
    """coefficients -> nodal E -> fused loss + adjoint -> dL/dcoefficients,
    against the oracle chain, then replayed as one CUDA graph."""
    torch = cuda
    from folax_gb300.batched import capture_step
    m = make_mesh("hex8", 8, seed=43)
    s = {"dirichlet_bc_dict": bc_dict("hex8", "elastic"), "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3},
         "control_layout": "nodal"}
    gl, ol = gpu_loss("hex8", "elastic", m, s), oracle_loss("hex8", "elastic", m, s)
    fc = _control(m)
    rng = np.random.default_rng(44)
    B = 2
    c = torch.tensor(0.5 * rng.standard_normal((B, fc.GetNumberOfVariables())), dtype=torch.float32, device="cuda")
    u = torch.tensor(0.01 * rng.standard_normal((B, gl.GetTotalNumberOfDOFs())), dtype=torch.float32, device="cuda")

    def step():
        E = fc.ComputeBatchControlledVariables(c)
        _, _, losses, du, dE = gl.ComputeBatchLossAndGrad(E, u)
        return losses, du, fc.ComputeBatchControlledVariablesVJP(c, dE)

    losses, du, dc = step()
    freqs = fo.fourier_frequencies(SETTINGS["x_freqs"], SETTINGS["y_freqs"], SETTINGS["z_freqs"])
    c64 = c.double().cpu().numpy()
    E_ref = fo.fourier_control_values(c64, freqs, _xyz(m), **_oracle_kw())
    _, _, l_ref, du_ref, dE_ref = ol.batch_loss_and_grads(E_ref, u.double().cpu().numpy())
    dc_ref = fo.fourier_control_vjp(c64, dE_ref, freqs, _xyz(m), **_oracle_kw())
    assert rel_fro(losses.cpu().numpy(), l_ref) < TOL
    assert rel_fro(du.cpu().numpy(), du_ref) < TOL
    assert rel_fro(dc.cpu().numpy(), dc_ref) < TOL
    graph, out = capture_step(step)
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(out[2], dc) and torch.equal(out[0], losses)
