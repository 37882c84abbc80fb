"""Seeded synthetic material fields (numpy.random.default_rng).

* fourier_conductivity: k = 0.1 + 0.9 * sigmoid(sum of 16 Fourier modes),
  wavenumbers 1..4, N(0,1) amplitudes, each mode a cos or a sin.
* two_phase_voxels: white noise on an n^3 voxel grid, Gaussian-smoothed
  (sigma in voxels, periodic FFT), thresholded at 0 -> E in {high, low}.
* FourierControl: the reference's nodal Fourier control
  (fol/controls/fourier_control.py:49-59) for parameter vectors.
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


class FourierControl:
    """Nodal Fourier control (fol/controls/fourier_control.py:14-62):
    K(x) = c0/2 + sum_f c_f cos(fx pi x) cos(fy pi y) cos(fz pi z),
    value = (max - min) * sigmoid(beta (K - 0.5)) + min."""

    def __init__(self, control_name: str, control_settings: dict, fe_mesh):
        self._name = control_name
        self.settings = control_settings
        self.fe_mesh = fe_mesh
        self.scale_min, self.scale_max = 0.0, 1.0

    def GetName(self):
        return self._name

    def Initialize(self, reinitialize=False):
        s = self.settings
        self.min = s.get("min", 1e-6)
        self.max = s.get("max", 1.0)
        self.beta = s["beta"]
        fx, fy, fz = (np.asarray(s[k]) for k in ("x_freqs", "y_freqs", "z_freqs"))
        mx, my, mz = np.meshgrid(fx, fy, fz, indexing="ij")
        self.frequencies = np.stack([mx.ravel(), my.ravel(), mz.ravel()], axis=1)
        self.num_control_vars = len(self.frequencies) + 1
        self.num_controlled_vars = self.fe_mesh.GetNumberOfNodes()

    def GetNumberOfVariables(self):
        return self.num_control_vars

    def GetNumberOfControlledVariables(self):
        return self.num_controlled_vars

    def ComputeControlledVariables(self, variable_vector):
        v = np.asarray(variable_vector, dtype=np.float64) * (self.scale_max - self.scale_min) + self.scale_min
        X = self.fe_mesh.GetNodesCoordinates()
        K = v[0] / 2.0 + np.zeros(len(X))
        for f, c in zip(self.frequencies, v[1:]):
            K += c * np.cos(f[0] * np.pi * X[:, 0]) * np.cos(f[1] * np.pi * X[:, 1]) * np.cos(f[2] * np.pi * X[:, 2])
        return (self.max - self.min) / (1.0 + np.exp(-self.beta * (K - 0.5))) + self.min

    def ComputeBatchControlledVariables(self, batch_variable_vector):
        return np.stack([self.ComputeControlledVariables(v) for v in np.atleast_2d(batch_variable_vector)])
