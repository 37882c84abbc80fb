"""folgb_loss_adjoint_noalloc: the fused loss + adjoint for callers that cannot
allocate device memory (it runs on a fixed scratch array inside the library).

Checked through the C ABI against folgb_loss_adjoint (caller workspace) on two
calls in a row, across two plans of different sizes that share the scratch,
and for the size limit.  Collected last on purpose: it leaves the shared
scratch in whatever state the last call wrote, which no other test reads.
"""
import ctypes as C

import numpy as np
import pytest

from gpu_cases import bc_dict, gpu_loss, make_mesh, rel_fro

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _call(torch, lib, loss, ctrl, u, noalloc):
    from folax_gb300 import _capi
    plan = loss._plan
    B = u.shape[0]
    P = torch.as_tensor(ctrl, dtype=torch.float32, device="cuda").contiguous()
    U = torch.as_tensor(u, dtype=torch.float32, device="cuda").contiguous()
    losses = torch.empty(B, dtype=torch.float32, device="cuda")
    du = torch.empty_like(U)
    dc = torch.empty((B, P.shape[1]), dtype=torch.float32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    cstride = 0 if P.shape[0] == 1 else P.shape[1]
    stream = _capi.stream_handle()
    if noalloc:
        rc = lib.folgb_loss_adjoint_noalloc(plan.handle, B, P.data_ptr(), cstride, U.data_ptr(), U.shape[1], 1,
                                            losses.data_ptr(), du.data_ptr(), dc.data_ptr(), status.data_ptr(),
                                            stream)
    else:
        nbytes = lib.folgb_workspace_bytes(plan.handle, _capi.OP_LOSS_ADJOINT, B)
        ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        rc = lib.folgb_loss_adjoint(plan.handle, B, P.data_ptr(), cstride, U.data_ptr(), U.shape[1], 1,
                                    losses.data_ptr(), du.data_ptr(), dc.data_ptr(), status.data_ptr(),
                                    ws.data_ptr(), C.c_size_t(nbytes), stream)
    torch.cuda.synchronize()
    return rc, int(status.item()), losses.cpu().numpy(), du.cpu().numpy(), dc.cpu().numpy()


def _case(etype, physics, n, layout, seed):
    m = make_mesh(etype, n, seed=seed)
    settings = {"dirichlet_bc_dict": bc_dict(etype, physics),
                "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3}, "control_layout": layout}
    return gpu_loss(etype, physics, m, settings)


def test_noalloc_matches_workspace_entry_point_on_two_calls(cuda):
    from folax_gb300 import _capi
    torch = cuda
    lib = _capi.load()
    big = _case("hex8", "elastic", 12, "element", seed=31)     # sum-factorised hex8 kernel
    small = _case("quad4", "thermal", 20, "nodal", seed=32)    # generic kernel, nodal control
    rng = np.random.default_rng(33)
    for call, loss in enumerate((big, small, big)):
        B = 2
        ctrl = 0.5 + rng.random((B, loss.GetNumberOfControls()))
        u = (0.03 / 12) * rng.standard_normal((B, loss.GetTotalNumberOfDOFs()))
        rc_n, st_n, *out_n = _call(torch, lib, loss, ctrl, u, noalloc=True)
        rc_w, st_w, *out_w = _call(torch, lib, loss, ctrl, u, noalloc=False)
        assert rc_n == _capi.OK and rc_w == _capi.OK, (call, rc_n, rc_w)
        assert st_n == 0 and st_w == 0
        for a, b in zip(out_n, out_w):
            assert rel_fro(a, b) < TOL, call


def test_noalloc_rejects_problems_larger_than_its_scratch(cuda):
    from folax_gb300 import _capi
    torch = cuda
    lib = _capi.load()
    loss = _case("hex8", "elastic", 16, "element", seed=34)
    B = 400  # 400 x 4096 elements x 32 floats: far above 48 MiB
    ctrl = np.ones((1, loss.GetNumberOfControls()))
    u = np.zeros((B, loss.GetTotalNumberOfDOFs()))
    rc, *_ = _call(torch, lib, loss, ctrl, u, noalloc=True)
    assert rc == _capi.ERR_TOO_LARGE


def test_noalloc_limit_covers_64cubed_hex8_and_rejects_one_instance_more(cuda):
    """The stated guarantee (64^3 hex8 elasticity, batch 1, fits the fixed
    scratch) for both control layouts, and the boundary: the largest batch
    that fits runs and matches the workspace entry point, one instance more
    is refused before any work."""
    from folax_gb300 import _capi
    from folax_gb300.loss import MechanicalLoss3DHexa
    from folax_gb300.mesh import create_3D_box_mesh
    torch = cuda
    lib = _capi.load()
    limit = 48 << 20
    m64 = create_3D_box_mesh(64, 64, 64)
    for layout in ("element", "nodal"):
        loss = MechanicalLoss3DHexa("l64", {"dirichlet_bc_dict": bc_dict("hex8", "elastic"),
                                            "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3},
                                            "control_layout": layout, "num_gp": 2}, m64)
        loss.Initialize()
        need = lib.folgb_workspace_bytes(loss._plan.handle, _capi.OP_LOSS_ADJOINT, 1)
        assert 0 < need <= limit, (layout, need)
        del loss
    loss = _case("hex8", "elastic", 16, "element", seed=35)
    ws = lambda b: lib.folgb_workspace_bytes(loss._plan.handle, _capi.OP_LOSS_ADJOINT, b)
    B = 1
    while ws(B + 1) <= limit:
        B += 1
    rng = np.random.default_rng(36)
    ctrl = 0.5 + rng.random((1, loss.GetNumberOfControls()))
    u = (0.03 / 16) * rng.standard_normal((B + 1, loss.GetTotalNumberOfDOFs()))
    rc, *_ = _call(torch, lib, loss, ctrl, u, noalloc=True)
    assert rc == _capi.ERR_TOO_LARGE
    rc_n, st_n, *out_n = _call(torch, lib, loss, ctrl, u[:B], noalloc=True)
    rc_w, st_w, *out_w = _call(torch, lib, loss, ctrl, u[:B], noalloc=False)
    assert rc_n == _capi.OK and rc_w == _capi.OK and st_n == 0 and st_w == 0
    for a, b in zip(out_n, out_w):
        assert rel_fro(a, b) < TOL
