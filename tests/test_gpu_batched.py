"""Many uneven instances in one persistent launch (C ABI folgb_batch_*),
the device Adam update, and CUDA-graph capture of the whole step."""
import numpy as np
import pytest

from gpu_cases import gpu_loss, rel_fro
from folax_gb300 import fields
from folax_gb300.mesh import create_2D_square_mesh, create_3D_box_mesh

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _instances(sizes, seed=0):
    meshes = [create_2D_square_mesh(1.0, n + 1) for n in sizes]
    rng = np.random.default_rng(seed)
    for m in meshes:
        m.nodes_coordinates = m.nodes_coordinates + (0.05 / (len(m.node_ids) ** 0.5)) * \
            rng.standard_normal(m.nodes_coordinates.shape) * np.array([1, 1, 0])
    return meshes


@pytest.mark.parametrize("layout,exponent", [("element", 1.0), ("nodal", 1.0), ("element", 1.5)])
def test_batched_matches_per_instance_launches(cuda, layout, exponent):
    from folax_gb300.batched import BatchedFELoss
    sizes = [5, 9, 3, 12, 7]
    meshes = _instances(sizes, seed=1)
    settings = {"dirichlet_bc_dict": {"T": {"left": 1.0, "right": 0.0}}, "control_layout": layout,
                "loss_function_exponent": exponent, "num_gp": 2}
    bl = BatchedFELoss("quad", "thermal", meshes, settings, elements_per_tile=16)
    rng = np.random.default_rng(2)
    ctrl_parts, u_parts = [], []
    for m in meshes:
        nc = len(m.elements_nodes["quad"]) if layout == "element" else m.GetNumberOfNodes()
        ctrl_parts.append(0.1 + rng.random(nc))
        u_parts.append(rng.random(m.GetNumberOfNodes()))
    mean, losses, du, dc = bl.ComputeLossAndGrad(np.concatenate(ctrl_parts), np.concatenate(u_parts))
    I = len(meshes)
    losses, du, dc = losses.cpu().numpy(), du.cpu().numpy(), dc.cpu().numpy()
    for i, m in enumerate(meshes):
        single = gpu_loss("quad4", "thermal", m, dict(settings))
        _, _, li, dui, dci = single.ComputeBatchLossAndGrad(ctrl_parts[i][None], u_parts[i][None])
        a, b = bl.dof_offsets[i], bl.dof_offsets[i + 1]
        c0, c1 = bl.control_offsets[i], bl.control_offsets[i + 1]
        assert rel_fro(losses[i], li.cpu().numpy()[0]) < TOL
        assert rel_fro(du[a:b] * I, dui.cpu().numpy()[0]) < TOL
        assert rel_fro(dc[c0:c1] * I, dci.cpu().numpy()[0]) < TOL
    assert abs(float(mean) - losses.mean()) <= 1e-6 * abs(losses.mean())


@pytest.mark.parametrize("n,offset", [(1000, 0), (1003, 0), (1000, 1)])
def test_adam_matches_reference_update(cuda, n, offset):
    """16-byte path (n a multiple of 4, aligned), its scalar tail (n = 1003)
    and the plain path (parameters starting 4 bytes into an allocation)."""
    torch = cuda
    from folax_gb300.batched import AdamState
    rng = np.random.default_rng(3)
    x0 = rng.standard_normal(n).astype(np.float32)
    x = torch.zeros(n + offset, device="cuda")[offset:]
    x.copy_(torch.tensor(x0, device="cuda"))
    st = AdamState(x, lr=1e-2)
    m = np.zeros_like(x0, dtype=np.float64)
    v = np.zeros_like(m)
    xr = x0.astype(np.float64)
    for t in range(1, 4):
        g = rng.standard_normal(n).astype(np.float32)
        st.update(x, torch.tensor(g, device="cuda"))
        m = 0.9 * m + 0.1 * g
        v = 0.999 * v + 0.001 * g.astype(np.float64) ** 2
        xr = xr - 1e-2 * (m / (1 - 0.9 ** t)) / (np.sqrt(v / (1 - 0.999 ** t)) + 1e-8)
    assert rel_fro(x.cpu().numpy() - x0, xr - x0) < 1e-4
    assert int(st.step.item()) == 3


def test_graph_captured_step_replays_exactly(cuda):
    """loss + adjoint + Adam captured once as a CUDA graph and replayed gives
    the same parameters as the same steps run eagerly."""
    torch = cuda
    from folax_gb300.batched import AdamState, BatchedFELoss, capture_step
    meshes = _instances([4, 6, 8], seed=4)
    settings = {"dirichlet_bc_dict": {"T": {"left": 1.0, "right": 0.0}}, "control_layout": "element", "num_gp": 2}
    bl = BatchedFELoss("quad", "thermal", meshes, settings, elements_per_tile=16)
    ctrl = torch.tensor(np.concatenate([0.1 + np.random.default_rng(5).random(len(m.elements_nodes["quad"]))
                                        for m in meshes]), dtype=torch.float32, device="cuda")
    T0 = torch.rand(bl.total_dofs, device="cuda")
    out = (torch.empty(bl.num_instances, device="cuda"), torch.empty_like(T0), torch.empty_like(ctrl))

    def run_eager(steps):
        T = T0.clone()
        st = AdamState(T, lr=1e-2)
        for _ in range(steps):
            _, _, du, _ = bl.ComputeLossAndGrad(ctrl, T, out=out)
            st.update(T, du)
        return T

    eager = run_eager(5)
    T = T0.clone()
    st = AdamState(T, lr=1e-2)

    def step():
        bl.ComputeLossAndGrad(ctrl, T, out=out)
        st.update(T, out[1])

    g, _ = capture_step(step, warmup=1)   # the warm-up step updates T once
    for _ in range(4):
        g.replay()
    torch.cuda.synchronize()
    assert int(st.step.item()) == 5
    assert torch.equal(T, eager)


def test_batch_autotune_keeps_a_tile_size_and_the_results(cuda):
    """The batched autotuner picks one of its tile sizes, leaves the plan on
    it, and the results stay those of the per-instance launches: gradients
    bit-identical to the untuned plan (the tile size does not enter them),
    losses within 1e-6 (summed in another grouping)."""
    torch = cuda
    from folax_gb300.batched import BatchedFELoss
    sizes = [40, 90, 17, 64, 128, 33]
    meshes = _instances(sizes, seed=7)
    settings = {"dirichlet_bc_dict": {"T": {"left": 1.0, "right": 0.0}}, "control_layout": "element", "num_gp": 2}
    bl = BatchedFELoss("quad", "thermal", meshes, settings, elements_per_tile=64)
    rng = np.random.default_rng(8)
    ctrl = torch.tensor(0.1 + rng.random(bl.num_elements), dtype=torch.float32, device="cuda")
    u = torch.tensor(rng.random(bl.total_dofs), dtype=torch.float32, device="cuda")
    _, l0, du0, dc0 = bl.ComputeLossAndGrad(ctrl, u)
    l0, du0, dc0 = l0.clone(), du0.clone(), dc0.clone()
    res = bl.Autotune(ctrl, u, repeats=2, cold_l2=False)
    assert res["chosen"] in BatchedFELoss.BATCH_TILES and bl.elements_per_tile == res["chosen"]
    assert len(res["ms"]) == len(BatchedFELoss.BATCH_TILES) and all(t > 0 for t in res["ms"])
    _, l1, du1, dc1 = bl.ComputeLossAndGrad(ctrl, u)
    assert torch.equal(du0, du1) and torch.equal(dc0, dc1)
    assert rel_fro(l1.cpu().numpy(), l0.cpu().numpy()) < 1e-6
    for i, m in enumerate(meshes):
        single = gpu_loss("quad4", "thermal", m, dict(settings))
        c0, c1 = bl.control_offsets[i], bl.control_offsets[i + 1]
        a, b = bl.dof_offsets[i], bl.dof_offsets[i + 1]
        _, _, li, _, _ = single.ComputeBatchLossAndGrad(ctrl[c0:c1][None], u[a:b][None])
        assert rel_fro(l1[i].cpu().numpy(), li.cpu().numpy()[0]) < TOL
