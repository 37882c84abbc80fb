"""ctypes binding of libfolgb.so (the C ABI declared in include/folgb.h).

The library is loaded from the package's ``lib/`` folder.  There is no CPU
fallback: if the library is missing or fails to load, every product entry
point raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_NONPOSITIVE_DETJ = 2
ERR_NAN = 3
ERR_NOT_CONVERGED = 4
ERR_CUDA = 5
ERR_WORKSPACE = 6
ERR_NO_PATTERN = 7
ERR_TOO_LARGE = 8
ERR_TIMEOUT = 9

STATUS_NAMES = {
    OK: "ok", ERR_INVALID_ARGUMENT: "invalid argument", ERR_NONPOSITIVE_DETJ: "non-positive detJ",
    ERR_NAN: "non-finite value", ERR_NOT_CONVERGED: "not converged", ERR_CUDA: "CUDA error",
    ERR_WORKSPACE: "workspace too small", ERR_NO_PATTERN: "plan has no CSR pattern",
    ERR_TOO_LARGE: "problem larger than the fixed scratch",
    ERR_TIMEOUT: "a bounded device-side wait gave up",
}

QUAD4, HEX8, TET4 = 0, 1, 2
THERMAL, ELASTIC, NEOHOOKE, SAINT_VENANT, TRANSIENT_THERMAL, NEOHOOKE_SPLIT = 0, 1, 2, 3, 4, 5
CONTROL_NODAL, CONTROL_ELEMENT = 0, 1
SHEAR_REFERENCE, SHEAR_CONSISTENT = 0, 1
OP_LOSS_ADJOINT, OP_ASSEMBLE, OP_PCG, OP_PLAIN, OP_KRYLOV64 = 0, 1, 2, 3, 4
KRYLOV_CG, KRYLOV_BICGSTAB = 0, 1
KRYLOV_ENGINE_GRID, KRYLOV_ENGINE_KERNELS = 0, 1
FEATURE_TILES, FEATURE_UNIFORM_BOX, FEATURE_BOX_GRID, FEATURE_TET_PATCHES = 1, 2, 4, 8


class FolgbError(RuntimeError):
    def __init__(self, func, code):
        super().__init__(f"{func} failed: {STATUS_NAMES.get(code, code)} (status {code})")
        self.code = code


class Monomial(C.Structure):
    _fields_ = [("coeff", C.c_double), ("control_power", C.c_int32), ("dof_power", C.c_int32 * 3)]


class Physics(C.Structure):
    _fields_ = [
        ("element_type", C.c_int32), ("physics", C.c_int32), ("num_gp", C.c_int32),
        ("control_layout", C.c_int32), ("shear_mode", C.c_int32), ("kernel_variant", C.c_int32),
        ("young_modulus", C.c_double), ("poisson_ratio", C.c_double),
        ("body_force", C.c_double * 3), ("beta", C.c_double), ("c", C.c_double),
        ("loss_exponent", C.c_double),
        ("rho_cp", C.c_double), ("time_step", C.c_double), ("material_beta", C.c_double),
    ]


class NewtonSettings(C.Structure):
    _fields_ = [("load_steps", C.c_int32), ("max_iterations", C.c_int32), ("abs_tol", C.c_double),
                ("rel_tol", C.c_double), ("krylov_method", C.c_int32), ("vector_bits", C.c_int32),
                ("krylov_rtol", C.c_double), ("krylov_maxiter", C.c_int32), ("check_every", C.c_int32),
                ("line_search", C.c_int32), ("line_search_max_halvings", C.c_int32)]


class NewtonInfo(C.Structure):
    _fields_ = [("newton_iterations", C.c_int32), ("krylov_iterations", C.c_int64), ("last_res_norm", C.c_double),
                ("last_delta_norm", C.c_double), ("krylov_failures", C.c_int32), ("status", C.c_int32),
                ("line_search_halvings", C.c_int32)]


vp = C.c_void_p
i32, i64, f32, f64, sz = C.c_int32, C.c_int64, C.c_float, C.c_double, C.c_size_t

# name -> (restype, argtypes)
PROTOTYPES = {
    "folgb_plan_create": (C.c_int, [C.POINTER(vp), C.POINTER(Physics), vp, i64, vp, i64, vp, vp, i64, i32]),
    "folgb_plan_destroy": (C.c_int, [vp]),
    "folgb_plan_info": (C.c_int, [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)]),
    "folgb_plan_features": (C.c_int, [vp, C.POINTER(C.c_int32)]),
    "folgb_plan_set_dirichlet_values": (C.c_int, [vp, vp, f64]),
    "folgb_plan_set_nodal_field": (C.c_int, [vp, vp]),
    "folgb_workspace_bytes": (sz, [vp, i32, i32]),
    "folgb_loss_adjoint": (C.c_int, [vp, i32, vp, i64, vp, i64, i32, vp, vp, vp, vp, vp, sz, vp]),
    "folgb_loss_adjoint_plain": (C.c_int, [vp, i32, vp, i64, vp, i64, i32, vp, vp, vp, vp, vp, sz, vp]),
    "folgb_loss_adjoint_noalloc": (C.c_int, [vp, i32, vp, i64, vp, i64, i32, vp, vp, vp, vp, vp]),
    "folgb_autotune": (C.c_int, [vp, i32, vp, i64, vp, i64, vp, vp, vp, vp, sz, i32, vp, C.POINTER(i32), vp, i32]),
    "folgb_autotune_flushed": (C.c_int, [vp, i32, vp, i64, vp, i64, vp, vp, vp, vp, sz, i32, vp, C.POINTER(i32), vp,
                                         i32, vp, sz]),
    "folgb_csr_pattern": (C.c_int, [vp, vp, vp, vp]),
    "folgb_assemble": (C.c_int, [vp, vp, vp, i32, vp, vp, vp, vp, vp, sz, vp]),
    "folgb_pcg": (C.c_int, [vp, vp, vp, vp, vp, f64, i32, i32, C.POINTER(i32), C.POINTER(f64), vp, sz, vp]),
    "folgb_bicgstab": (C.c_int, [vp, vp, vp, vp, vp, f64, i32, i32, C.POINTER(i32), C.POINTER(f64), vp, sz, vp]),
    "folgb_krylov": (C.c_int, [vp, i32, i32, vp, vp, vp, vp, f64, i32, i32, C.POINTER(i32), C.POINTER(f64), vp, sz,
                               vp]),
    "folgb_krylov_set_engine": (C.c_int, [i32]),
    "folgb_krylov_async": (C.c_int, [vp, i32, i32, vp, vp, vp, vp, f64, i32, i32, vp, vp, vp, vp, sz, vp]),
    "folgb_spmv": (C.c_int, [vp, vp, vp, vp, vp]),
    "folgb_newton_workspace_bytes": (sz, [vp, C.POINTER(NewtonSettings)]),
    "folgb_newton": (C.c_int, [vp, vp, vp, C.POINTER(NewtonSettings), C.POINTER(NewtonInfo), vp, vp, vp, sz, vp]),
    "folgb_adam_step": (C.c_int, [vp, vp, vp, vp, i64, vp, f32, f32, f32, f32, vp]),
    "folgb_batch_plan_create": (C.c_int, [C.POINTER(vp), C.POINTER(Physics), i32, vp, vp, vp, vp, vp, vp, i64, i32]),
    "folgb_batch_plan_destroy": (C.c_int, [vp]),
    "folgb_batch_workspace_bytes": (sz, [vp]),
    "folgb_batch_loss_adjoint": (C.c_int, [vp, vp, vp, i32, vp, vp, vp, vp, vp, sz, vp]),
    "folgb_batch_autotune": (C.c_int, [vp, vp, vp, i32, vp, vp, vp, vp, vp, sz, i32, vp, sz, vp, C.POINTER(i32), vp,
                                       i32]),
    "folgb_response_workspace_bytes": (sz, [vp]),
    "folgb_response": (C.c_int, [vp, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, sz, vp]),
    "folgb_fourier_create": (C.c_int, [C.POINTER(vp), vp, i32, vp, i32, vp, i32, vp, i64, f64, f64, f64, f64, f64]),
    "folgb_fourier_destroy": (C.c_int, [vp]),
    "folgb_fourier_forward": (C.c_int, [vp, i32, vp, vp, vp]),
    "folgb_fourier_workspace_bytes": (sz, [vp, i32]),
    "folgb_fourier_backward": (C.c_int, [vp, i32, vp, vp, vp, vp, sz, vp]),
    "folgb_selftest_bounded_wait": (C.c_int, [vp, vp]),
    "folgb_fp32_peak_probe": (C.c_int, [vp, i32, i32, C.POINTER(f64), vp]),
    "folgb_trace_enable": (C.c_int, [i32]),
    "folgb_trace_reset": (C.c_int, []),
    "folgb_trace_read": (C.c_int, [i32, C.POINTER(i64), C.POINTER(f64)]),
}

KERNEL_IDS = {"elem_loss": 0, "gather": 1, "elem_matrix": 2, "pair_reduce": 3, "plain_backward": 4,
              "elem_residual": 5, "pcg_spmv": 6, "pcg_update": 7, "batch_loss": 8, "hex8_fused": 9}

_LIB = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libfolgb.so (building it first when it is missing or stale)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if build_if_missing and (_build.needs_build()):
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libfolgb.so not found at {path}; run folax_gb300.build.build()")
    lib = C.CDLL(path)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(func: str, code: int):
    if code != OK:
        raise FolgbError(func, code)


def ptr(t) -> int | None:
    """Device (or host) address of a torch tensor / numpy array, or None."""
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    return t.ctypes.data


_RAW_STREAM = None


def stream_handle(stream=None) -> int:
    """cudaStream_t of `stream`, or of torch's current stream on the current
    device (through torch's raw-stream query when it has one: ~0.2 us instead
    of ~3 us for building a Stream object on every call)."""
    global _RAW_STREAM
    import torch
    if stream is not None:
        return stream.cuda_stream
    if _RAW_STREAM is None:
        raw = getattr(torch._C, "_cuda_getCurrentRawStream", None)
        _RAW_STREAM = (lambda: raw(torch.cuda.current_device())) if raw is not None else \
            (lambda: torch.cuda.current_stream().cuda_stream)
    return _RAW_STREAM()
