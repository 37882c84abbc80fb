"""Many parametric instances with uneven meshes in one persistent launch.

The reference batches instances of ONE mesh (fol/loss_functions/fe_loss.py:
250-262, a vmap over the batch).  Operator-learning data sets of different
domain sizes need many meshes; ``BatchedFELoss`` concatenates them into one
plan with per-instance offset tables (include/folgb.h:
folgb_batch_plan_create) so a single persistent kernel evaluates every
instance's loss and adjoint, and ``AdamState`` applies the optimiser update
(optax.adam semantics, deep_network.py:100,141) on the device.
``capture_step`` records loss + adjoint + update as one CUDA graph;
``BatchedFELoss.Autotune`` picks the elements per tile of the launch.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi as capi
from .loss import _ETYPE, _dev, _torch

_PHYSICS = {"thermal": capi.THERMAL, "elastic": capi.ELASTIC, "neohooke": capi.NEOHOOKE,
            "saint_venant": capi.SAINT_VENANT}
_NDOF = {("quad", "thermal"): 1, ("hexahedron", "thermal"): 1, ("tetra", "thermal"): 1,
         ("quad", "elastic"): 2, ("hexahedron", "elastic"): 3, ("tetra", "elastic"): 3,
         ("quad", "neohooke"): 2, ("hexahedron", "neohooke"): 3, ("tetra", "neohooke"): 3,
         ("quad", "saint_venant"): 2, ("hexahedron", "saint_venant"): 3, ("tetra", "saint_venant"): 3}


class BatchedFELoss:
    """Fused loss + adjoint over a list of meshes (one element type and physics).

    meshes: list of Mesh; settings: the reference's loss_settings keys
    (dirichlet_bc_dict, material_dict, num_gp, control_layout, ...), applied to
    every instance.  Controls and dofs are concatenated over instances in mesh
    order (``control_offsets`` / ``dof_offsets``)."""

    def __init__(self, element_type: str, physics: str, meshes, settings: dict, elements_per_tile: int = 1024):
        self.lib = capi.load()
        self.element_type, self.physics_name = element_type, physics
        self.settings = settings
        self.meshes = meshes
        self.elements_per_tile = int(elements_per_tile)
        ndof = _NDOF[(element_type, physics)]
        self.ndof = ndof
        dofnames = ["T"] if ndof == 1 else ["Ux", "Uy", "Uz"][:ndof]
        conn, xyz, eoff, noff, didx, dval = [], [], [0], [0], [], []
        for m in meshes:
            c = np.asarray(m.GetElementsNodes(element_type), dtype=np.int64)
            x = np.asarray(m.GetNodesCoordinates(), dtype=np.float64)
            x3 = np.zeros((len(x), 3))
            x3[:, : x.shape[1]] = x
            for di, dof in enumerate(dofnames):
                for set_name, value in settings["dirichlet_bc_dict"].get(dof, {}).items():
                    nodes = np.asarray(m.GetNodeSet(set_name), dtype=np.int64)
                    didx.append(ndof * (noff[-1] + nodes) + di)
                    dval.append(np.full(len(nodes), float(value)))
            conn.append(c)
            xyz.append(x3)
            eoff.append(eoff[-1] + len(c))
            noff.append(noff[-1] + len(x))
        self.element_offsets = np.asarray(eoff, dtype=np.int64)
        self.node_offsets = np.asarray(noff, dtype=np.int64)
        self.num_instances = len(meshes)
        self.num_elements = int(eoff[-1])
        self.num_nodes = int(noff[-1])
        self.total_dofs = ndof * self.num_nodes
        layout = settings.get("control_layout", "nodal")
        self.control_offsets = self.element_offsets if layout == "element" else self.node_offsets
        self.dof_offsets = ndof * self.node_offsets
        self.dirichlet_indices = np.concatenate(didx) if didx else np.zeros(0, np.int64)
        self.dirichlet_values = np.concatenate(dval) if dval else np.zeros(0)
        conn_all = np.ascontiguousarray(np.concatenate(conn))
        xyz_all = np.ascontiguousarray(np.concatenate(xyz))
        mat = settings.get("material_dict", {})
        p = capi.Physics()
        p.element_type = _ETYPE[element_type]
        p.physics = _PHYSICS[physics]
        p.num_gp = int(settings.get("num_gp", 1 if element_type == "tetra" else 2))
        p.control_layout = capi.CONTROL_ELEMENT if layout == "element" else capi.CONTROL_NODAL
        p.shear_mode = capi.SHEAR_CONSISTENT if settings.get("voigt_shear_mode") == "consistent" else capi.SHEAR_REFERENCE
        p.kernel_variant = 0
        p.young_modulus = float(mat.get("young_modulus", 1.0))
        p.poisson_ratio = float(mat.get("poisson_ratio", 0.3))
        bf = np.zeros(3)
        if "body_foce" in settings and physics != "thermal":
            b = np.asarray(settings["body_foce"], dtype=np.float64).ravel()
            bf[: len(b)] = b
        p.body_force[0], p.body_force[1], p.body_force[2] = bf
        p.beta = float(settings.get("beta", 0.0))
        p.c = float(settings.get("c", 1.0))
        p.loss_exponent = float(settings.get("loss_function_exponent", 1.0))
        _torch().cuda.init()
        h = C.c_void_p()
        di = np.ascontiguousarray(self.dirichlet_indices)
        dv = np.ascontiguousarray(self.dirichlet_values)
        rc = self.lib.folgb_batch_plan_create(C.byref(h), C.byref(p), self.num_instances,
                                              self.element_offsets.ctypes.data, self.node_offsets.ctypes.data,
                                              conn_all.ctypes.data, xyz_all.ctypes.data,
                                              di.ctypes.data if len(di) else None,
                                              dv.ctypes.data if len(dv) else None, len(di), int(elements_per_tile))
        capi.check("folgb_batch_plan_create", rc)
        self.handle = h
        torch = _torch()
        nbytes = int(self.lib.folgb_batch_workspace_bytes(h))
        self.workspace = torch.empty(max(nbytes, 256), dtype=torch.uint8, device="cuda")
        self.status = torch.zeros(1, dtype=torch.int32, device="cuda")

    def ComputeLossAndGrad(self, control, dofs, out=None):
        """Returns (mean, per-instance losses, dLoss/d dofs, dLoss/d control);
        the gradients are of the mean over instances."""
        torch = _torch()
        ctrl = _dev(control).reshape(-1)
        u = _dev(dofs).reshape(-1)
        if out is None:
            losses = torch.empty(self.num_instances, dtype=torch.float32, device="cuda")
            du = torch.empty_like(u)
            dc = torch.empty_like(ctrl)
        else:
            losses, du, dc = out
        rc = self.lib.folgb_batch_loss_adjoint(self.handle, capi.ptr(ctrl), capi.ptr(u), 1, capi.ptr(losses),
                                               capi.ptr(du), capi.ptr(dc), capi.ptr(self.status),
                                               capi.ptr(self.workspace), self.workspace.numel(), capi.stream_handle())
        capi.check("folgb_batch_loss_adjoint", rc)
        return losses.mean(), losses, du, dc

    BATCH_TILES = (256, 512, 1024, 2048, 4096)

    def Autotune(self, control, dofs, repeats: int = 5, cold_l2: bool = True):
        """Times the batched launch with each tile size of BATCH_TILES
        (elements per tile) on these inputs and keeps the fastest in the plan
        (folgb_batch_autotune); cold_l2: a temporary 256 MiB device buffer is
        overwritten before every timed call, as inside a training step.
        Returns {"chosen": elements per tile, "ms": [per-size times]}."""
        torch = _torch()
        ctrl = _dev(control).reshape(-1)
        u = _dev(dofs).reshape(-1)
        losses = torch.empty(self.num_instances, dtype=torch.float32, device="cuda")
        du, dc = torch.empty_like(u), torch.empty_like(ctrl)
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda") if cold_l2 else None
        chosen = C.c_int32()
        times = (C.c_float * len(self.BATCH_TILES))()
        rc = self.lib.folgb_batch_autotune(self.handle, capi.ptr(ctrl), capi.ptr(u), 1, capi.ptr(losses), capi.ptr(du),
                                           capi.ptr(dc), capi.ptr(self.status), capi.ptr(self.workspace),
                                           self.workspace.numel(), int(repeats),
                                           capi.ptr(flush) if flush is not None else None,
                                           flush.numel() if flush is not None else 0, capi.stream_handle(),
                                           C.byref(chosen), C.cast(times, C.c_void_p), len(self.BATCH_TILES))
        del flush
        capi.check("folgb_batch_autotune", rc)
        self.elements_per_tile = chosen.value
        return {"chosen": chosen.value, "ms": [times[i] for i in range(len(self.BATCH_TILES))]}

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.lib.folgb_batch_plan_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


class AdamState:
    """Adam moments and step counter on the device (optax.adam defaults)."""

    def __init__(self, params, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        torch = _torch()
        self.lib = capi.load()
        self.m = torch.zeros_like(params)
        self.v = torch.zeros_like(params)
        self.step = torch.zeros(1, dtype=torch.int32, device="cuda")
        self.lr, self.beta1, self.beta2, self.eps = lr, beta1, beta2, eps

    def update(self, params, grads):
        rc = self.lib.folgb_adam_step(capi.ptr(params), capi.ptr(grads), capi.ptr(self.m), capi.ptr(self.v),
                                      params.numel(), capi.ptr(self.step), self.lr, self.beta1, self.beta2, self.eps,
                                      capi.stream_handle())
        capi.check("folgb_adam_step", rc)


def shard_instances(element_counts, world_size: int):
    """Instances of a batch spread over world_size ranks (one GPU each) by
    element count: largest instance first onto the least-loaded rank (ties to
    the lower rank), so every rank gets about the same number of elements.
    Instances are independent, so the ranks exchange nothing on the data
    path; only the scalar loss mean needs one reduction.  Returns one
    ascending index array per rank; deterministic."""
    counts = np.asarray(element_counts, dtype=np.int64)
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    load = np.zeros(world_size, dtype=np.int64)
    parts = [[] for _ in range(world_size)]
    for i in sorted(range(len(counts)), key=lambda k: (-counts[k], k)):
        r = int(np.argmin(load))  # first minimum: the lowest rank among ties
        parts[r].append(i)
        load[r] += counts[i]
    return [np.asarray(sorted(p), dtype=np.int64) for p in parts]


def capture_step(fn, warmup: int = 3):
    """Record fn() (device work only, fixed buffers) as a CUDA graph; returns
    (graph, result of the captured call).  Replaying the graph repeats the work."""
    torch = _torch()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(warmup):
            fn()
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        res = fn()
    return g, res
