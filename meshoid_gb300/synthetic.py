"""Seeded synthetic particle sets and fields (NumPy, FP64).

The reference's own walkthrough runs on a downloaded simulation snapshot that
is not available offline; these generators stand in for it with the particle
distributions the benchmark workloads are defined on:

* ``uniform``       -- N points uniform in [0, 1)^3.
* ``plummer``       -- Plummer sphere, scale a, radii truncated at r_max*a,
                       isotropic directions, equal masses.
* ``clump_mixture`` -- 64 Gaussian clumps (centres uniform in [-1,1]^3,
                       widths log-uniform in [1e-3, 1e-1], Dirichlet(1)
                       weights) plus a 20% uniform background in [-1,1]^3.
* ``fourier_fields`` -- scalar fields, each a sum of 8 random Fourier modes
                       A sin(2 pi k.x + phi) with integer wave vectors,
                       |k| in [1, 32].
* ``rotation_velocity`` -- solid-body rotation Omega x r plus N(0, sigma) noise.
"""
from __future__ import annotations

import numpy as np


def uniform(n: int, seed: int = 0, dim: int = 3) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.random((n, dim))


def _isotropic(rng, n):
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1)[:, None]
    return v


def plummer(n: int, seed: int = 0, a: float = 1.0, r_max: float = 20.0) -> np.ndarray:
    """Plummer radii r = a / sqrt(u^(-2/3) - 1), rejection-truncated at r <= r_max*a."""
    rng = np.random.default_rng(seed)
    out = np.empty((0,), dtype=np.float64)
    while out.size < n:
        u = rng.random(int((n - out.size) * 1.05) + 16)
        u = np.clip(u, 1e-300, 1.0 - 1e-16)
        r = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        out = np.concatenate([out, r[r <= r_max * a]])
    r = out[:n]
    return r[:, None] * _isotropic(rng, n)


def clump_mixture(n: int, seed: int = 0, n_clumps: int = 64, background: float = 0.2,
                  sigma_range=(1e-3, 1e-1)) -> np.ndarray:
    rng = np.random.default_rng(seed)
    n_bg = int(round(background * n))
    n_cl = n - n_bg
    centres = rng.uniform(-1.0, 1.0, size=(n_clumps, 3))
    sig = np.exp(rng.uniform(np.log(sigma_range[0]), np.log(sigma_range[1]), size=n_clumps))
    w = rng.dirichlet(np.ones(n_clumps))
    counts = rng.multinomial(n_cl, w)
    parts = [rng.uniform(-1.0, 1.0, size=(n_bg, 3))]
    for c in range(n_clumps):
        if counts[c]:
            parts.append(centres[c] + sig[c] * rng.normal(size=(counts[c], 3)))
    pos = np.concatenate(parts, axis=0)
    return pos[rng.permutation(n)]


def fourier_modes(n_fields: int, seed: int = 0, n_modes: int = 8, kmax: int = 32):
    """Per field, n_modes (k, amplitude, phase): k integer with 1 <= |k| <= kmax,
    amplitude N(0, 1) / |k|, phase U[0, 2 pi)."""
    rng = np.random.default_rng(seed)
    modes = []
    for _ in range(n_fields):
        fm = []
        for _ in range(n_modes):
            while True:
                k = rng.integers(-kmax, kmax + 1, size=3)
                nk = np.linalg.norm(k)
                if 1.0 <= nk <= kmax:
                    break
            amp = rng.normal() / max(nk, 1.0)
            phi = rng.uniform(0, 2 * np.pi)
            fm.append((k, amp, phi))
        modes.append(fm)
    return modes


def fourier_fields(pos: np.ndarray, n_fields: int, seed: int = 0, n_modes: int = 8,
                   kmax: int = 32) -> np.ndarray:
    """(N, n_fields) FP64: each field sums n_modes terms A sin(2 pi k.x + phi)."""
    out = np.zeros((pos.shape[0], n_fields))
    for f, fm in enumerate(fourier_modes(n_fields, seed, n_modes, kmax)):
        for k, amp, phi in fm:
            out[:, f] += amp * np.sin(2 * np.pi * (pos @ k) + phi)
    return out


def fourier_fields_torch(pos, n_fields: int, seed: int = 0, n_modes: int = 8, kmax: int = 32):
    """fourier_fields evaluated in FP64 by torch on pos's device (same modes)."""
    import torch
    out = torch.zeros((pos.shape[0], n_fields), dtype=torch.float64, device=pos.device)
    for f, fm in enumerate(fourier_modes(n_fields, seed, n_modes, kmax)):
        for k, amp, phi in fm:
            kk = torch.as_tensor(k.astype(np.float64), device=pos.device)
            out[:, f] += amp * torch.sin(2 * np.pi * (pos @ kk) + phi)
    return out


def rotation_velocity(pos: np.ndarray, omega=(0.0, 0.0, 1.0), sigma: float = 0.1,
                      seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.cross(np.asarray(omega, dtype=np.float64)[None, :], pos) + rng.normal(0.0, sigma, size=pos.shape)


def config1_field(pos: np.ndarray) -> np.ndarray:
    """sin(2 pi x) cos(2 pi y) + z^2, the first-order D test field of the small uniform workload."""
    return np.sin(2 * np.pi * pos[:, 0]) * np.cos(2 * np.pi * pos[:, 1]) + pos[:, 2] ** 2
