"""FE loss classes: the reference's FiniteElementLoss API over libfolgb.so.

Mirrors fol/loss_functions/fe_loss.py:19-318 and its subclasses
(thermal.py, mechanical.py, mechanical_neohooke_AD.py): the same class names,
constructor arguments (name, loss_settings, fe_mesh), settings keys and
methods.  Arrays go to the GPU as float32 torch tensors; every numerical step
runs in the CUDA kernels behind include/folgb.h.  There is no CPU path.

Differences a caller can see:
* ComputeBatchLossAndGrad returns the gradients jax.grad would give for the
  dofs, and the true derivative of the loss value for the control (the
  reference's jax.grad wrt the control is 0 for the stop_gradient losses,
  mechanical.py:116, thermal.py:45-49).
* loss_settings["control_layout"] = "element" takes one control value per
  element (de = value * 1); the default "nodal" gathers nodal controls by
  connectivity as the reference does.
* ComputeJacobianMatrixAndResidualVector returns a CSRJacobian (canonical CSR,
  the pattern scipy.sparse.csr_array builds from the reference's BCOO).
* The kernels report a non-positive detJ, a non-finite value or a device wait
  that gave up through a status word on the GPU.  A wait that gave up makes
  every output of that call invalid.  loss_settings["check_device_status"] =
  True reads the word after every call (one stream synchronisation) and
  raises FolgbError before any result is returned; otherwise call
  CheckDeviceStatus() where a check is wanted.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _capi as capi
from .mesh import Mesh

_ETYPE = {"quad": capi.QUAD4, "hexahedron": capi.HEX8, "tetra": capi.TET4}
# sum-factorised hex8 kernel variants (threads per block x accumulation scheme)
HEX8_VARIANTS = 25
HEX8_VARIANT_NAMES = ["256 thr, point sums", "128 thr, point sums", "256 thr, dual coefficients",
                      "128 thr, dual coefficients", "64 thr, point sums", "64 thr, dual coefficients",
                      "128 thr, 96 regs, point sums", "128 thr, 96 regs, dual coefficients",
                      "128 thr, 80 regs, point sums", "128 thr, 80 regs, dual coefficients",
                      "256 thr, paired points (f32x2)", "128 thr, paired points (f32x2)",
                      "128 thr, 96 regs, paired points (f32x2)",
                      "persistent, TMA-staged rows, paired points (f32x2)",
                      "persistent, TMA-staged rows, 96 regs, paired points (f32x2)",
                      "persistent, TMA-staged rows, 96 regs, point sums",
                      "persistent, TMA-staged rows, next tile's nodes prefetched to L1, paired points (f32x2)",
                      "persistent, TMA-staged rows, next tile's nodes prefetched to L2, paired points (f32x2)",
                      "tile-local, persistent: tile inputs copied ahead by cp.async, residuals summed in shared "
                      "memory, paired points (f32x2)",
                      "tile-local, one block per tile, paired points (f32x2)",
                      "uniform box: 3x3 blocks of the element matrix in the Hadamard basis, persistent, "
                      "TMA-staged rows",
                      "uniform box: 3x3 blocks of the element matrix in the Hadamard basis, 256 thr",
                      "uniform box: 3x3 blocks of the element matrix in the Hadamard basis, 128 thr",
                      "structured box grid: one launch, no records, 16x8 node columns, layer chunks for one wave",
                      "structured box grid: one launch, no records, 16x8 node columns, layer chunks for two waves"]
_NEN = {"quad": 4, "hexahedron": 8, "tetra": 4}


def _torch():
    import torch
    return torch


def _dev(x, dtype=None):
    torch = _torch()
    dtype = dtype or torch.float32
    if isinstance(x, torch.Tensor):
        if x.is_cuda and x.dtype == dtype and x.is_contiguous():
            return x  # already usable: no conversion call on the hot path
        if x.device.type == "cpu" and x.is_pinned() and x.dtype == dtype and x.is_contiguous():
            return x.to(device="cuda", non_blocking=True)  # stream-ordered copy from pinned memory
        return x.to(device="cuda", dtype=dtype).contiguous()
    return torch.as_tensor(np.asarray(x), dtype=dtype, device="cuda").contiguous()


class Plan:
    """Owns one folgb_plan (mesh tables on the device) and cached workspaces."""

    def __init__(self, phys: capi.Physics, conn: np.ndarray, xyz: np.ndarray, dir_idx: np.ndarray,
                 dir_val: np.ndarray, build_csr: bool):
        self.lib = capi.load()
        conn = np.ascontiguousarray(conn, dtype=np.int64)
        xyz3 = np.zeros((len(xyz), 3))
        xyz = np.asarray(xyz, dtype=np.float64)
        xyz3[:, : xyz.shape[1]] = xyz
        di = np.ascontiguousarray(dir_idx, dtype=np.int64)
        dv = np.ascontiguousarray(dir_val, dtype=np.float64)
        self.phys = phys
        h = C.c_void_p()
        _torch().cuda.init()
        rc = self.lib.folgb_plan_create(C.byref(h), C.byref(phys), conn.ctypes.data, len(conn), xyz3.ctypes.data,
                                        len(xyz3), di.ctypes.data if len(di) else None,
                                        dv.ctypes.data if len(dv) else None, len(di), int(build_csr))
        capi.check("folgb_plan_create", rc)
        self.handle = h
        nd, tot, rows, nnz = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        capi.check("folgb_plan_info", self.lib.folgb_plan_info(h, C.byref(nd), C.byref(tot), C.byref(rows),
                                                                C.byref(nnz)))
        self.ndof, self.total_dofs, self.rows, self.nnz = nd.value, tot.value, rows.value, nnz.value
        self.num_elements = len(conn)
        self.num_nodes = len(xyz3)
        self.has_csr = bool(build_csr)
        self._ws = {}
        self._ws_fit = {}  # (op, batch) -> a buffer known to be large enough
        self._pattern = None

    def workspace(self, op: int, batch: int = 1):
        buf = self._ws_fit.get((op, batch))
        if buf is not None:
            return buf
        torch = _torch()
        n = int(self.lib.folgb_workspace_bytes(self.handle, op, batch))
        buf = self._ws.get(op)
        if buf is None or buf.numel() < n:
            buf = torch.empty(max(n, 256), dtype=torch.uint8, device="cuda")
            self._ws[op] = buf
            self._ws_fit = {k: v for k, v in self._ws_fit.items() if k[0] != op}
        self._ws_fit[(op, batch)] = buf
        return buf

    def set_dirichlet_values(self, values: np.ndarray, load_increment: float = 1.0):
        v = np.ascontiguousarray(values, dtype=np.float64)
        capi.check("folgb_plan_set_dirichlet_values",
                   self.lib.folgb_plan_set_dirichlet_values(self.handle, v.ctypes.data if len(v) else None,
                                                            float(load_increment)))

    def pattern(self):
        """Canonical CSR pattern (indptr, indices) as int32 device tensors."""
        torch = _torch()
        if self._pattern is None:
            indptr = torch.empty(self.rows + 1, dtype=torch.int32, device="cuda")
            indices = torch.empty(self.nnz, dtype=torch.int32, device="cuda")
            capi.check("folgb_csr_pattern", self.lib.folgb_csr_pattern(self.handle, capi.ptr(indptr),
                                                                        capi.ptr(indices), capi.stream_handle()))
            self._pattern = (indptr, indices)
        return self._pattern

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.lib.folgb_plan_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


@dataclass
class CSRJacobian:
    """BC-applied Jacobian in canonical CSR form (device tensors)."""
    indptr: object
    indices: object
    data: object
    inv_diag: object
    shape: tuple
    plan: Plan

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_array((self.data.double().cpu().numpy(), self.indices.cpu().numpy(),
                             self.indptr.cpu().numpy()), shape=self.shape)

    def to_torch(self):
        torch = _torch()
        return torch.sparse_csr_tensor(self.indptr, self.indices, self.data, size=self.shape)

    def todense(self):
        return self.to_scipy().toarray()

    def matvec(self, x):
        torch = _torch()
        x = _dev(x)
        y = torch.empty_like(x)
        capi.check("folgb_spmv", self.plan.lib.folgb_spmv(self.plan.handle, capi.ptr(self.data), capi.ptr(x),
                                                          capi.ptr(y), capi.stream_handle()))
        return y


class FiniteElementLoss:
    """fe_loss.py:19-318 over the GB300 kernels."""

    physics = None  # set by subclasses

    def __init__(self, name: str, loss_settings: dict, fe_mesh: Mesh):
        self._name = name
        self.loss_settings = loss_settings
        self.dofs = loss_settings["ordered_dofs"]
        self.element_type = loss_settings["element_type"]
        self.fe_mesh = fe_mesh
        self.initialized = False
        if "dirichlet_bc_dict" not in loss_settings:
            raise ValueError("dirichlet_bc_dict should provided in the loss settings !")

    def GetName(self):
        return self._name

    # fe_loss.py:34-55
    def _create_dofs_dict(self):
        n = len(self.dofs)
        idx, val = [], []
        for di, dof in enumerate(self.dofs):
            for set_name, value in self.loss_settings["dirichlet_bc_dict"].get(dof, {}).items():
                nodes = np.asarray(self.fe_mesh.GetNodeSet(set_name), dtype=np.int64)
                idx.append(n * nodes + di)
                val.append(float(value) * np.ones(len(nodes)))
        self.dirichlet_indices = np.concatenate(idx) if idx else np.zeros(0, np.int64)
        self.dirichlet_values = np.concatenate(val) if val else np.zeros(0)
        all_idx = np.arange(n * self.fe_mesh.GetNumberOfNodes())
        self.non_dirichlet_indices = np.setdiff1d(all_idx, self.dirichlet_indices)

    def _physics_struct(self) -> capi.Physics:
        s = self.loss_settings
        mat = s.get("material_dict", {})
        p = capi.Physics()
        p.element_type = _ETYPE[self.element_type]
        p.physics = self.physics
        p.num_gp = int(self.num_gp)
        p.control_layout = capi.CONTROL_ELEMENT if s.get("control_layout", "nodal") == "element" else capi.CONTROL_NODAL
        p.shear_mode = capi.SHEAR_CONSISTENT if s.get("voigt_shear_mode", "reference") == "consistent" else capi.SHEAR_REFERENCE
        kv = s.get("kernel_variant", "auto")
        p.kernel_variant = 1 if kv == "generic" else (2 + int(kv) if isinstance(kv, int) else 0)
        p.young_modulus = float(mat.get("young_modulus", 1.0))
        p.poisson_ratio = float(mat.get("poisson_ratio", 0.3))
        bf = np.zeros(3)
        if "body_foce" in s and self.physics != capi.THERMAL:
            b = np.asarray(s["body_foce"], dtype=np.float64).ravel()
            bf[: len(b)] = b
        p.body_force[0], p.body_force[1], p.body_force[2] = bf
        p.beta = float(getattr(self, "_beta", 0.0))
        p.c = float(getattr(self, "_c", 1.0))
        p.loss_exponent = float(self.loss_function_exponent)
        p.rho_cp = float(getattr(self, "_rho_cp", 1.0))
        p.time_step = float(getattr(self, "_dt", 1.0))
        p.material_beta = float(getattr(self, "_mbeta", 0.0))
        return p

    def _configure_plan(self, plan: "Plan") -> "Plan":
        """Per-plan data beyond the physics struct (overridden where needed)."""
        return plan

    def Initialize(self, reinitialize=False) -> None:
        if self.initialized and not reinitialize:
            return
        s = self.loss_settings
        self.number_dofs_per_node = len(self.dofs)
        self.total_number_of_dofs = len(self.dofs) * self.fe_mesh.GetNumberOfNodes()
        self._create_dofs_dict()
        self.number_of_unknown_dofs = self.non_dirichlet_indices.size
        # fe_loss.py:68-83 (order 1 when unset)
        self.num_gp = int(s.get("num_gp", 1))
        s["num_gp"] = self.num_gp
        if self.num_gp not in (1, 2, 3):
            raise ValueError(f" number gauss points {self.num_gp} is not supported ! ")
        if "compute_dims" not in s:
            raise ValueError(f"compute_dims must be provided in the loss settings of {self.GetName()}! ")
        self.dim = s["compute_dims"]
        self.loss_function_exponent = float(s.get("loss_function_exponent", 1.0))
        self.parametric_boundary_learning = bool(s.get("parametric_boundary_learning", False))
        conn = np.asarray(self.fe_mesh.GetElementsNodes(self.element_type), dtype=np.int64)
        xyz = np.asarray(self.fe_mesh.GetNodesCoordinates(), dtype=np.float64)
        self._conn, self._xyz = conn, xyz
        self._plan = self._configure_plan(Plan(self._physics_struct(), conn, xyz, self.dirichlet_indices,
                                               self.dirichlet_values, False))
        self._csr_plan = None
        self._status = _torch().zeros(1, dtype=_torch().int32, device="cuda")
        self._strict_status = bool(s.get("check_device_status", False))
        # the last call's validated arguments (ComputeBatchLossAndGrad); the
        # epoch changes whenever the plan's kernel path may have changed
        self._memo = None
        self._epoch = getattr(self, "_epoch", 0) + 1
        self.initialized = True

    def _get_csr_plan(self) -> Plan:
        if self._csr_plan is None:
            self._csr_plan = self._configure_plan(Plan(self._physics_struct(), self._conn, self._xyz,
                                                       self.dirichlet_indices, self.dirichlet_values, True))
        return self._csr_plan

    def Finalize(self) -> None:
        pass

    def GetNumberOfUnknowns(self):
        return self.number_of_unknown_dofs

    def GetTotalNumberOfDOFs(self):
        return self.total_number_of_dofs

    def GetDOFs(self):
        return self.dofs

    def GetNumberOfControls(self):
        if self.loss_settings.get("control_layout", "nodal") == "element":
            return self.fe_mesh.GetNumberOfElements(self.element_type)
        return self.fe_mesh.GetNumberOfNodes()

    def GetDeviceStatus(self) -> int:
        """Status bits raised by the kernels (1 << FOLGB_ERR_*); reading it synchronises."""
        return int(self._status.item())

    def KernelFeatures(self) -> dict:
        """Kernel paths this mesh allows: "tiles" (tile-local hex8 kernels),
        "uniform_box" (every element the same axis-aligned box: the box
        kernels, variants 20-22) and "box_grid" (also numbered as a structured
        box mesh: the one-launch grid kernels, variants 23-24, loss exponent
        1; a call with host result buffers runs the box kernel and the gather
        instead) and "tet_patches" (every 6 consecutive tetrahedra on at most
        8 nodes, as the 6-tet split of hexahedra: the loss + adjoint of
        3-component mechanics writes one record per group node; the
        "generic" kernel_variant turns it off).  The autotuner times the
        hex8 variants that apply."""
        f = C.c_int32()
        capi.check("folgb_plan_features", self._plan.lib.folgb_plan_features(self._plan.handle, C.byref(f)))
        return {"tiles": bool(f.value & capi.FEATURE_TILES), "uniform_box": bool(f.value & capi.FEATURE_UNIFORM_BOX),
                "box_grid": bool(f.value & capi.FEATURE_BOX_GRID),
                "tet_patches": bool(f.value & capi.FEATURE_TET_PATCHES)}

    def CheckDeviceStatus(self):
        """Raise FolgbError if a kernel flagged a non-positive detJ, a
        non-finite value or a device wait that gave up, then clear the flags."""
        st = self.GetDeviceStatus()
        self._status.zero_()
        for code in (capi.ERR_NONPOSITIVE_DETJ, capi.ERR_NAN, capi.ERR_TIMEOUT):
            if (st >> code) & 1:
                raise capi.FolgbError("FE kernel", code)

    # fe_loss.py:91-100, 124-125
    def GetFullDofVector(self, known_dofs, unknown_dofs):
        torch = _torch()
        full = _dev(unknown_dofs).clone()
        squeeze = full.dim() == 1
        if squeeze:
            full = full[None]
        idx = torch.as_tensor(self.dirichlet_indices, device="cuda")
        if self.parametric_boundary_learning:
            full[:, idx] = _dev(known_dofs).reshape(full.shape[0], -1)
        else:
            full[:, idx] = torch.as_tensor(self.dirichlet_values, dtype=torch.float32, device="cuda")
        return full[0] if squeeze else full

    # fe_loss.py:186-189
    def ApplyDirichletBCOnDofVector(self, full_dof_vector, load_increment: float = 1.0):
        torch = _torch()
        u = _dev(full_dof_vector).clone()
        idx = torch.as_tensor(self.dirichlet_indices, device="cuda")
        u[..., idx] = torch.as_tensor(load_increment * self.dirichlet_values, dtype=torch.float32, device="cuda")
        return u

    def _batched(self, batch_params, batch_dofs):
        P = _dev(batch_params)
        U = _dev(batch_dofs)
        U = U.reshape(-1, self.total_number_of_dofs) if U.dim() != 2 else U
        if U.shape[1] != self.total_number_of_dofs:
            raise ValueError(f"dofs must have {self.total_number_of_dofs} entries per instance")
        ncontrol = self.GetNumberOfControls()
        P = P.reshape(-1, ncontrol)
        B = U.shape[0]
        if P.shape[0] not in (1, B):
            raise ValueError("batch_params must have 1 or batch rows")
        return P, U, B

    def ComputeBatchLossAndGrad(self, batch_params, batch_dofs, grads: bool = True, plain: bool = False,
                                out=None):
        """Fused FE loss + adjoint (fe_loss.py:250-262 and its reverse pass).

        Returns (mean, (min, max, mean), per-instance losses, dLoss/d dofs,
        dLoss/d params); the gradients are None when grads is False.

        Host buffers: out = (losses [B], dLoss/d dofs [B, dofs],
        dLoss/d params [B, controls]) gives the result buffers, float32 and
        contiguous, on the GPU or in pinned host memory.  The kernels store the
        gradients straight into pinned host buffers over the host link (no
        separate device-to-host copy) and the per-instance losses follow with
        one small copy; like torch's non_blocking copies, host results are
        complete once the current stream has finished (mean / min / max stay
        on the GPU).  Pinned host inputs: the dofs are copied to the GPU on the
        current stream; element-layout controls (read once per element) are
        read by the kernel straight from pinned host memory.  A call with the
        same tensors as the previous one reuses its validated arguments."""
        torch = _torch()
        key = self._call_key(torch, batch_params, batch_dofs, grads, plain, out)
        memo = self._memo
        if key is not None and memo is not None and memo[0] == key:
            prep = memo[1]  # the same tensors as the last call, all used in place: no re-validation
        else:
            prep, in_place = self._prepare_call(torch, batch_params, batch_dofs, grads, plain, out)
            self._memo = (key, prep) if (key is not None and in_place) else None
        return self._run_call(torch, prep)

    def _call_key(self, torch, batch_params, batch_dofs, grads, plain, out):
        """Identity of a call's tensors (object, data pointer, shape) or None."""
        if not (isinstance(batch_params, torch.Tensor) and isinstance(batch_dofs, torch.Tensor)):
            return None
        k = [self._epoch, grads, plain]
        for t in (batch_params, batch_dofs) + (tuple(out) if out is not None else ()):
            if not isinstance(t, torch.Tensor):
                return None
            k += [id(t), t.data_ptr(), tuple(t.shape)]
        return tuple(k)

    def _prepare_call(self, torch, batch_params, batch_dofs, grads, plain, out):
        """Validated arguments of a loss + adjoint call, and whether every
        input is used in place (no converted copy, so a later call with the
        same tensors may reuse them)."""
        direct_ctrl = (isinstance(batch_params, torch.Tensor) and batch_params.device.type == "cpu"
                       and batch_params.is_pinned() and batch_params.dtype == torch.float32
                       and batch_params.is_contiguous() and self._plan.phys.control_layout == capi.CONTROL_ELEMENT
                       and not self.parametric_boundary_learning)
        # host tensors are copied to the GPU on every call (into buffers kept
        # with the prepared call); element controls in pinned memory are read
        # by the kernel in place
        copies = []

        def staged(t):
            if isinstance(t, torch.Tensor) and t.device.type == "cpu":
                d = torch.empty(t.shape, dtype=torch.float32, device="cuda")
                copies.append((d, t))
                d.copy_(t, non_blocking=True)
                return d
            return _dev(t)

        U = staged(batch_dofs)
        U = U.reshape(-1, self.total_number_of_dofs) if U.dim() != 2 else U
        if direct_ctrl:
            if U.shape[1] != self.total_number_of_dofs:
                raise ValueError(f"dofs must have {self.total_number_of_dofs} entries per instance")
            P, B = batch_params.reshape(-1, self.GetNumberOfControls()), U.shape[0]
            if P.shape[0] not in (1, B):
                raise ValueError("batch_params must have 1 or batch rows")
        else:
            P, U, B = self._batched(staged(batch_params), U)
        used = {t.data_ptr() for t in (batch_params, batch_dofs) if isinstance(t, torch.Tensor)}
        used |= {d.data_ptr() for d, _ in copies}
        in_place = (isinstance(batch_params, torch.Tensor) and isinstance(batch_dofs, torch.Tensor)
                    and P.data_ptr() in used and U.data_ptr() in used)
        apply_bc = 1
        if self.parametric_boundary_learning:
            U = self.GetFullDofVector(P, U)
            apply_bc = 0
            in_place = False
        out_losses = du = dp = None
        if out is not None:
            out_losses, du, dp = out
            want = [(out_losses, (B,)), (du, (B, U.shape[1])), (dp, (B, P.shape[1]))]
            for t, shape in want:
                if (t.dtype != torch.float32 or not t.is_contiguous() or t.numel() != int(np.prod(shape))
                        or not (t.is_cuda or t.is_pinned())):
                    raise ValueError(f"out buffers must be float32, contiguous, of {shape} elements, "
                                     "on the GPU or in pinned host memory")
        op = capi.OP_PLAIN if plain else capi.OP_LOSS_ADJOINT
        ws = self._plan.workspace(op, B)
        fn = self._plan.lib.folgb_loss_adjoint_plain if plain else self._plan.lib.folgb_loss_adjoint
        prep = {"P": P, "U": U, "B": B, "apply_bc": apply_bc, "out_losses": out_losses, "du": du, "dp": dp,
                "grads": grads, "plain": plain, "ws": ws, "fn": fn, "copies": copies, "fresh": True,
                "args": (capi.ptr(P), 0 if P.shape[0] == 1 else P.shape[1], capi.ptr(U), U.shape[1], apply_bc)}
        return prep, in_place

    def _run_call(self, torch, prep):
        B, out_losses = prep["B"], prep["out_losses"]
        if not prep["fresh"]:  # the host inputs, copied again for this call
            for d, t in prep["copies"]:
                d.copy_(t, non_blocking=True)
        prep["fresh"] = False
        if out_losses is not None:
            du, dp = prep["du"], prep["dp"]
            losses = out_losses if out_losses.is_cuda else torch.empty(B, dtype=torch.float32, device="cuda")
        else:
            losses = torch.empty(B, dtype=torch.float32, device="cuda")
            U, P = prep["U"], prep["P"]
            du = torch.empty(U.shape, dtype=torch.float32, device="cuda") if prep["grads"] else None
            dp = torch.empty((B, P.shape[1]), dtype=torch.float32, device="cuda") if prep["grads"] else None
        ws = prep["ws"]
        rc = prep["fn"](self._plan.handle, B, *prep["args"], capi.ptr(losses), capi.ptr(du), capi.ptr(dp),
                        capi.ptr(self._status), capi.ptr(ws), ws.numel(), capi.stream_handle())
        capi.check("folgb_loss_adjoint_plain" if prep["plain"] else "folgb_loss_adjoint", rc)
        if self._strict_status:
            self.CheckDeviceStatus()
        if out_losses is not None and out_losses is not losses:
            out_losses.copy_(losses, non_blocking=True)
        ret_losses = losses if out_losses is None else out_losses
        if B == 1:  # views, no extra kernels
            mean = losses[0]
            return mean, (mean, mean, mean), ret_losses, du, dp
        mean = losses.mean()
        return mean, (losses.min(), losses.max(), mean), ret_losses, du, dp

    def Autotune(self, batch_params, batch_dofs, repeats: int = 5, cold_l2: bool = True):
        """Time the plan's kernel variants on these inputs and keep the fastest.
        cold_l2: every timed call starts with the L2 cache flushed (a
        temporary 256 MiB device buffer is overwritten before it,
        folgb_autotune_flushed), as inside a training step; otherwise the calls
        run back to back (folgb_autotune).  Returns {"chosen": v, "ms":
        [per-variant times]}."""
        torch = _torch()
        P, U, B = self._batched(batch_params, batch_dofs)
        losses = torch.empty(B, dtype=torch.float32, device="cuda")
        du = torch.empty_like(U)
        dp = torch.empty((B, P.shape[1]), dtype=torch.float32, device="cuda")
        ws = self._plan.workspace(capi.OP_LOSS_ADJOINT, B)
        chosen = C.c_int32()
        times = (C.c_float * HEX8_VARIANTS)()
        args = (self._plan.handle, B, capi.ptr(P), 0 if P.shape[0] == 1 else P.shape[1], capi.ptr(U), U.shape[1],
                capi.ptr(losses), capi.ptr(du), capi.ptr(dp), capi.ptr(ws), ws.numel(), repeats,
                capi.stream_handle(), C.byref(chosen), C.cast(times, C.c_void_p), HEX8_VARIANTS)
        if cold_l2:
            flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
            rc = self._plan.lib.folgb_autotune_flushed(*args, capi.ptr(flush), flush.numel())
            del flush
            capi.check("folgb_autotune_flushed", rc)
        else:
            rc = self._plan.lib.folgb_autotune(*args)
            capi.check("folgb_autotune", rc)
        tunable = (self.element_type == "hexahedron" and self.physics == capi.ELASTIC and self.num_gp == 2
                   and self.loss_settings.get("kernel_variant", "auto") == "auto")
        n = HEX8_VARIANTS if tunable else 1
        self._memo = None  # the kernel path (and whether host dofs are read in place) may have changed
        self._epoch += 1
        return {"chosen": chosen.value, "ms": [times[i] for i in range(n)]}

    def ComputeBatchLoss(self, batch_params, batch_dofs):
        mean, stats, _, _, _ = self.ComputeBatchLossAndGrad(batch_params, batch_dofs, grads=False)
        return mean, stats

    def ComputeTotalEnergy(self, total_control_vars, total_primal_vars):
        """Sum of element energies for one instance (fe_loss.py:175-176); the
        dofs are used as given (no Dirichlet overwrite)."""
        torch = _torch()
        P, U, B = self._batched(total_control_vars, total_primal_vars)
        losses = torch.empty(B, dtype=torch.float32, device="cuda")
        ws = self._plan.workspace(capi.OP_LOSS_ADJOINT, B)
        # a plan with exponent != 1 would raise the sum to p; the energy is p = 1
        if self.loss_function_exponent != 1.0:
            raise NotImplementedError("ComputeTotalEnergy with loss_function_exponent != 1")
        rc = self._plan.lib.folgb_loss_adjoint(self._plan.handle, B, capi.ptr(P), 0 if P.shape[0] == 1 else P.shape[1],
                                               capi.ptr(U), U.shape[1], 0, capi.ptr(losses), None, None,
                                               capi.ptr(self._status), capi.ptr(ws), ws.numel(), capi.stream_handle())
        capi.check("folgb_loss_adjoint", rc)
        return losses[0] if B == 1 else losses

    # fe_loss.py:264-318
    def ComputeJacobianMatrixAndResidualVector(self, total_control_vars, total_primal_vars,
                                               transpose_jacobian: bool = False, with_matrix: bool = True):
        torch = _torch()
        # the residual alone needs no CSR tables
        plan = self._get_csr_plan() if with_matrix else self._plan
        ctrl = _dev(total_control_vars).reshape(-1)
        u = _dev(total_primal_vars).reshape(-1)
        residual = torch.empty(self.total_number_of_dofs, dtype=torch.float32, device="cuda")
        data = torch.empty(plan.nnz, dtype=torch.float32, device="cuda") if with_matrix else None
        inv_diag = torch.empty(self.total_number_of_dofs, dtype=torch.float32, device="cuda") if with_matrix else None
        ws = plan.workspace(capi.OP_ASSEMBLE)
        rc = plan.lib.folgb_assemble(plan.handle, capi.ptr(ctrl), capi.ptr(u), int(bool(transpose_jacobian)),
                                     capi.ptr(residual), capi.ptr(data), capi.ptr(inv_diag), capi.ptr(self._status),
                                     capi.ptr(ws), ws.numel(), capi.stream_handle())
        capi.check("folgb_assemble", rc)
        if self._strict_status:
            self.CheckDeviceStatus()
        if not with_matrix:
            return None, residual
        indptr, indices = plan.pattern()
        n = self.total_number_of_dofs
        return CSRJacobian(indptr, indices, data, inv_diag, (n, n), plan), residual

    def ComputeElement(self, xyze, de, uvwe):
        """One element's (energy, residual, stiffness) through the GPU kernels
        (the element API of fe_loss.py:143-147), as float64 numpy arrays."""
        xyze = np.asarray(xyze, dtype=np.float64)
        nen = _NEN[self.element_type]
        de = np.asarray(de, dtype=np.float64).reshape(-1)
        ue = np.asarray(uvwe, dtype=np.float64).reshape(-1)
        mesh = Mesh("element", "element.mem")
        mesh.node_ids = np.arange(nen)
        mesh.nodes_coordinates = xyze
        mesh.elements_nodes = {self.element_type: np.arange(nen)[None]}
        settings = dict(self.loss_settings)
        settings["dirichlet_bc_dict"] = {d: {} for d in self.dofs}
        settings["loss_function_exponent"] = 1.0
        settings["control_layout"] = "nodal"
        one = type(self)(self._name + "_element", settings, mesh)
        one.Initialize()
        jac, res = one.ComputeJacobianMatrixAndResidualVector(de, ue)
        en = one.ComputeTotalEnergy(de, ue)
        return float(en.item()), res.double().cpu().numpy(), jac.todense()


# ---------------------------------------------------------------------------
# element physics (class names and defaults of the reference)
# ---------------------------------------------------------------------------

def _with(loss_settings, **kw):
    return {**loss_settings, **kw}


class ThermalLoss(FiniteElementLoss):
    """thermal.py:14-49: k_gp = (N.de)(1 + beta (N.T)^c); energy T.sg(Se T - Fe)."""
    physics = capi.THERMAL

    def Initialize(self, reinitialize=False) -> None:
        self._beta = float(self.loss_settings.get("beta", 0.0))
        self._c = float(self.loss_settings.get("c", 1.0))
        super().Initialize(reinitialize)


class ThermalLoss2DQuad(ThermalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        loss_settings.setdefault("num_gp", 2)
        super().__init__(name, _with(loss_settings, compute_dims=2, ordered_dofs=["T"], element_type="quad"), fe_mesh)


class ThermalLoss3DHexa(ThermalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        loss_settings.setdefault("num_gp", 2)
        super().__init__(name, _with(loss_settings, compute_dims=3, ordered_dofs=["T"], element_type="hexahedron"),
                         fe_mesh)


class ThermalLoss3DTetra(ThermalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        super().__init__(name, _with(loss_settings, compute_dims=3, ordered_dofs=["T"], element_type="tetra"), fe_mesh)


class MechanicalLoss(FiniteElementLoss):
    """mechanical.py:13-117: Se = sum w detJ (N.de) B^T D B; energy u.sg(Se u - Fe)."""
    physics = capi.ELASTIC

    def Initialize(self, reinitialize=False) -> None:
        if "material_dict" not in self.loss_settings:
            raise ValueError("material_dict should provided in the loss settings !")
        super().Initialize(reinitialize)


class MechanicalLoss3DHexa(MechanicalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        loss_settings.setdefault("num_gp", 2)
        super().__init__(name, _with(loss_settings, compute_dims=3, ordered_dofs=["Ux", "Uy", "Uz"],
                                     element_type="hexahedron"), fe_mesh)


class MechanicalLoss3DTetra(MechanicalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        super().__init__(name, _with(loss_settings, compute_dims=3, ordered_dofs=["Ux", "Uy", "Uz"],
                                     element_type="tetra"), fe_mesh)


class MechanicalLoss2DQuad(MechanicalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        loss_settings.setdefault("num_gp", 2)
        super().__init__(name, _with(loss_settings, compute_dims=2, ordered_dofs=["Ux", "Uy"], element_type="quad"),
                         fe_mesh)


class NeoHookeMechanicalLoss(FiniteElementLoss):
    """mechanical_neohooke_AD.py:18-293: energy sum w detJ psi(C); residual
    B^T S_voigt - Fe with the reference's doubled-shear S_voigt unless
    loss_settings["voigt_shear_mode"] = "consistent"."""
    physics = capi.NEOHOOKE

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


class SaintVenantMechanicalLoss(FiniteElementLoss):
    """mechanical_saint_venant.py:18-296: Saint-Venant-Kirchhoff, energy
    sum w detJ psi(E) (psi = lam/2 tr(E)^2 + mu E:E, Lame constants from the
    Young's modulus control), residual B(F)^T S - Fe, tangent B^T C B plus the
    geometric stiffness."""
    physics = capi.SAINT_VENANT

    def Initialize(self, reinitialize=False) -> None:
        if "material_dict" not in self.loss_settings:
            raise ValueError("material_dict should provided in the loss settings !")
        super().Initialize(reinitialize)


class SaintVenantMechanicalLoss3DTetra(SaintVenantMechanicalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        super().__init__(name, _with(loss_settings, compute_dims=3, ordered_dofs=["Ux", "Uy", "Uz"],
                                     element_type="tetra"), fe_mesh)


class SaintVenantMechanicalLoss3DHexa(SaintVenantMechanicalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        loss_settings.setdefault("num_gp", 2)
        super().__init__(name, _with(loss_settings, compute_dims=3, ordered_dofs=["Ux", "Uy", "Uz"],
                                     element_type="hexahedron"), fe_mesh)


class SaintVenantMechanicalLoss2DQuad(SaintVenantMechanicalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        loss_settings.setdefault("num_gp", 2)
        super().__init__(name, _with(loss_settings, compute_dims=2, ordered_dofs=["Ux", "Uy"], element_type="quad"),
                         fe_mesh)


class TransientThermalLoss(ThermalLoss):
    """transient_thermal.py:16-172: implicit-Euler step of nonlinear heat
    conduction.  The control is the CURRENT nodal temperature field, the dofs
    the NEXT one; material_dict gives rho, cp, beta and the nodal conductivity
    k0 (default ones), time_integration_dict the time step, loss_settings "c"
    the exponent of K = k0 (1 + beta T^c).  Energy (the loss) is
    1/2 T.Se(T).T + rho cp/(2 dt) |T - T_current|^2 per element, with its true
    gradient; the residual (Me + dt Se) T - Me T_current and the tangent
    Me + dt Se_dR follow transient_thermal.py:64-78."""
    physics = capi.TRANSIENT_THERMAL

    def Initialize(self, reinitialize=False) -> None:
        if self.initialized and not reinitialize:
            return
        mat = {"rho": 1.0, "cp": 1.0, "beta": 0.0, **self.loss_settings.get("material_dict", {})}
        ti = {"method": "implicit-euler", "time_step": None, **self.loss_settings.get("time_integration_dict", {})}
        if ti["time_step"] is None:
            raise ValueError("time step should be provided in the time_integration_dict ")
        n = self.fe_mesh.GetNumberOfNodes()
        k0 = np.asarray(mat.get("k0", np.ones(n)), dtype=np.float64).reshape(-1)
        if k0.shape != (n,):
            raise ValueError(f"provided k0({k0.shape}) in the material_dict does not match the mesh with {n} nodes !")
        self._k0 = np.ascontiguousarray(k0)
        self._rho_cp = float(mat["rho"]) * float(mat["cp"])
        self._dt = float(ti["time_step"])
        self._mbeta = float(mat["beta"])
        self.loss_settings["control_layout"] = "nodal"
        super().Initialize(reinitialize)
        self._beta = 0.0

    def _configure_plan(self, plan):
        capi.check("folgb_plan_set_nodal_field", plan.lib.folgb_plan_set_nodal_field(plan.handle,
                                                                                    self._k0.ctypes.data))
        return plan

    def ComputeElement(self, xyze, Te_c, Te_n, Ke):
        """(energy, residual, tangent) of one element (transient_thermal.py:43-78)."""
        nen = _NEN[self.element_type]
        settings = dict(self.loss_settings)
        settings["material_dict"] = {**settings.get("material_dict", {}),
                                     "k0": np.asarray(Ke, dtype=np.float64).reshape(nen)}
        xyze = np.asarray(xyze, dtype=np.float64)
        mesh = Mesh("element", "element.mem")
        mesh.node_ids = np.arange(nen)
        mesh.nodes_coordinates = xyze
        mesh.elements_nodes = {self.element_type: np.arange(nen)[None]}
        settings["dirichlet_bc_dict"] = {d: {} for d in self.dofs}
        settings["loss_function_exponent"] = 1.0
        one = type(self)(self._name + "_element", settings, mesh)
        one.Initialize()
        tc = np.asarray(Te_c, dtype=np.float64).reshape(-1)
        tn = np.asarray(Te_n, dtype=np.float64).reshape(-1)
        jac, res = one.ComputeJacobianMatrixAndResidualVector(tc, tn)
        en = one.ComputeTotalEnergy(tc, tn)
        return float(en.item()), res.double().cpu().numpy(), jac.todense()


class TransientThermalLoss3DTetra(TransientThermalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        super().__init__(name, _with(loss_settings, compute_dims=3, ordered_dofs=["T"], element_type="tetra"), fe_mesh)


class TransientThermalLoss3DHexa(TransientThermalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        loss_settings.setdefault("num_gp", 2)
        super().__init__(name, _with(loss_settings, compute_dims=3, ordered_dofs=["T"], element_type="hexahedron"),
                         fe_mesh)


class TransientThermalLoss2DQuad(TransientThermalLoss):
    def __init__(self, name, loss_settings, fe_mesh):
        loss_settings.setdefault("num_gp", 2)
        super().__init__(name, _with(loss_settings, compute_dims=2, ordered_dofs=["T"], element_type="quad"), fe_mesh)
