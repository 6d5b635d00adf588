"""Shared helpers for the GPU parity tests (tolerances live in the tests)."""
import numpy as np


def as_np(t):
    try:
        import torch
        if isinstance(t, torch.Tensor):
            return t.detach().double().cpu().numpy() if t.is_floating_point() else t.detach().cpu().numpy()
    except ImportError:
        pass
    return np.asarray(t)


def sets_equal_rows(a, b):
    """Row-wise set equality of neighbour index arrays; returns the mismatching row count."""
    a = np.sort(np.asarray(a), axis=1)
    b = np.sort(np.asarray(b), axis=1)
    return int(np.sum(np.any(a != b, axis=1)))


def row_rel_err(got, ref, floor_frac=1e-3):
    """Per-row ||got - ref|| / max(||ref||, floor_frac * median ||ref||)."""
    got = np.asarray(got, dtype=np.float64).reshape(len(got), -1)
    ref = np.asarray(ref, dtype=np.float64).reshape(len(ref), -1)
    scale = np.linalg.norm(ref, axis=1)
    floor = floor_frac * max(np.median(scale), 1e-300)
    return np.linalg.norm(got - ref, axis=1) / np.maximum(scale, floor)


def summary(err):
    err = np.asarray(err)
    return f"max {err.max():.3g} rms {np.sqrt(np.mean(err ** 2)):.3g}"
