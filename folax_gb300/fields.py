"""Seeded synthetic material fields (numpy.random.default_rng).

* fourier_conductivity: k = 0.1 + 0.9 * sigmoid(sum of 16 Fourier modes),
  wavenumbers 1..4, N(0,1) amplitudes, each mode a cos or a sin.
* two_phase_voxels: white noise on an n^3 voxel grid, Gaussian-smoothed
  (sigma in voxels, periodic FFT), thresholded at 0 -> E in {high, low}.
* FourierControl: the reference's nodal Fourier control
  (fol/controls/fourier_control.py:14-59), evaluated on the device by
  folgb_fourier_forward / folgb_fourier_backward (no host round trip).
"""
from __future__ import annotations

import numpy as np


def fourier_conductivity(points: np.ndarray, seed: int, n_modes: int = 16, kmax: int = 4,
                         kmin_val: float = 0.1, span: float = 0.9) -> np.ndarray:
    rng = np.random.default_rng(seed)
    amp = rng.standard_normal(n_modes)
    kx = rng.integers(1, kmax + 1, n_modes)
    ky = rng.integers(1, kmax + 1, n_modes)
    use_sin = rng.integers(0, 2, n_modes).astype(bool)
    x, y = points[:, 0], points[:, 1]
    s = np.zeros(len(points))
    for m in range(n_modes):
        arg = 2.0 * np.pi * (kx[m] * x + ky[m] * y)
        s += amp[m] * (np.sin(arg) if use_sin[m] else np.cos(arg))
    return kmin_val + span / (1.0 + np.exp(-s))


def two_phase_voxels(n: int, seed: int, sigma: float = 3.0, high: float = 1.0, low: float = 0.1) -> np.ndarray:
    """Voxel field (n^3,) in element order (x fastest, then y, then z)."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((n, n, n))
    f = np.fft.fftfreq(n)
    gz, gy, gx = np.meshgrid(f, f, f, indexing="ij")
    kernel = np.exp(-2.0 * (np.pi * sigma) ** 2 * (gx ** 2 + gy ** 2 + gz ** 2))
    sm = np.real(np.fft.ifftn(np.fft.fftn(w) * kernel))
    return np.where(sm > 0.0, high, low).ravel()


def element_centroids(xyz: np.ndarray, conn: np.ndarray) -> np.ndarray:
    return xyz[conn].mean(axis=1)


class IdentityControl:
    """fol/controls/identity_control.py: the controlled variables are the
    control variables (a nodal or element field given directly)."""

    def __init__(self, control_name: str, control_settings: dict, num_vars: int):
        self._name = control_name
        self.settings = control_settings
        self.num_vars = int(num_vars)
        self.initialized = False

    def GetName(self):
        return self._name

    def Initialize(self, reinitialize=False):
        self.num_control_vars = self.num_vars
        self.num_controlled_vars = self.num_vars
        self.initialized = True

    def GetNumberOfVariables(self):
        return self.num_vars

    def GetNumberOfControlledVariables(self):
        return self.num_vars

    def ComputeControlledVariables(self, variable_vector):
        from .loss import _dev
        return _dev(variable_vector)

    def ComputeBatchControlledVariables(self, batch_variable_vector):
        from .loss import _dev
        return _dev(batch_variable_vector).reshape(-1, self.num_vars)


class FourierControl:
    """Nodal Fourier control (fol/controls/fourier_control.py:14-59):
    K(x) = v0/2 + sum_f v_f cos(fx pi x) cos(fy pi y) cos(fz pi z),
    value = (max - min) * sigmoid(beta (K - 0.5)) + min, with
    v = coeffs * (scale_max - scale_min) + scale_min.  Evaluated on the GPU;
    results are CUDA tensors."""

    def __init__(self, control_name: str, control_settings: dict, fe_mesh):
        self._name = control_name
        self.settings = control_settings
        self.fe_mesh = fe_mesh
        self.scale_min, self.scale_max = 0.0, 1.0
        self.initialized = False
        self._handle = None
        self._ws = {}

    def GetName(self):
        return self._name

    def Initialize(self, reinitialize=False):
        if self.initialized and not reinitialize:
            return
        import ctypes as C
        from . import _capi as capi
        s = self.settings
        self.min = float(s.get("min", 1e-6))
        self.max = float(s.get("max", 1.0))
        self.beta = float(s["beta"])
        self.x_freqs, self.y_freqs, self.z_freqs = (np.atleast_1d(np.asarray(s[k], dtype=np.float64))
                                                    for k in ("x_freqs", "y_freqs", "z_freqs"))
        self.num_control_vars = len(self.x_freqs) * len(self.y_freqs) * len(self.z_freqs) + 1
        self.num_controlled_vars = self.fe_mesh.GetNumberOfNodes()
        self.lib = capi.load()
        X = np.asarray(self.fe_mesh.GetNodesCoordinates(), dtype=np.float64)
        xyz = np.zeros((len(X), 3))
        xyz[:, : X.shape[1]] = X
        xyz = np.ascontiguousarray(xyz)
        self._destroy()
        h = C.c_void_p()
        capi.check("folgb_fourier_create", self.lib.folgb_fourier_create(
            C.byref(h), self.x_freqs.ctypes.data, len(self.x_freqs), self.y_freqs.ctypes.data, len(self.y_freqs),
            self.z_freqs.ctypes.data, len(self.z_freqs), xyz.ctypes.data, len(xyz), self.min, self.max, self.beta,
            float(self.scale_min), float(self.scale_max)))
        self._handle = h
        self.initialized = True

    def GetNumberOfVariables(self):
        return self.num_control_vars

    def GetNumberOfControlledVariables(self):
        return self.num_controlled_vars

    def _coeffs(self, batch_variable_vector):
        import torch
        from .loss import _dev
        c = _dev(batch_variable_vector).reshape(-1, self.num_control_vars)
        return c, torch

    def ComputeBatchControlledVariables(self, batch_variable_vector):
        """(B, F+1) coefficients -> (B, N) nodal values (CUDA tensor)."""
        from . import _capi as capi
        c, torch = self._coeffs(batch_variable_vector)
        out = torch.empty((c.shape[0], self.num_controlled_vars), dtype=torch.float32, device="cuda")
        capi.check("folgb_fourier_forward", self.lib.folgb_fourier_forward(
            self._handle, c.shape[0], capi.ptr(c), capi.ptr(out), capi.stream_handle()))
        return out

    def ComputeControlledVariables(self, variable_vector):
        return self.ComputeBatchControlledVariables(variable_vector)[0]

    def ComputeBatchControlledVariablesVJP(self, batch_variable_vector, batch_dvalues):
        """d(sum dvalues * values) / d coefficients, (B, F+1) (CUDA tensor):
        the gradient jax.grad propagates through the control."""
        from . import _capi as capi
        from .loss import _dev
        c, torch = self._coeffs(batch_variable_vector)
        g = _dev(batch_dvalues).reshape(c.shape[0], self.num_controlled_vars)
        B = c.shape[0]
        ws = self._ws.get(B)
        if ws is None:
            n = int(self.lib.folgb_fourier_workspace_bytes(self._handle, B))
            ws = self._ws[B] = torch.empty(max(n, 256), dtype=torch.uint8, device="cuda")
        out = torch.empty_like(c)
        capi.check("folgb_fourier_backward", self.lib.folgb_fourier_backward(
            self._handle, B, capi.ptr(c), capi.ptr(g), capi.ptr(out), capi.ptr(ws), ws.numel(),
            capi.stream_handle()))
        return out

    def _destroy(self):
        if getattr(self, "_handle", None):
            self.lib.folgb_fourier_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self._destroy()
        except Exception:
            pass
