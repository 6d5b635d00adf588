"""Learned first guess of the smoothing length (the "seed network").

A 54 -> 64 -> 64 -> 1 MLP (GELU, bf16 weights, FP32 accumulation) maps the
log2(1 + count) occupancy of the 27 cells around a particle at the next finer
level and at its adaptive level (the finest level whose cell around the
particle holds >= max(2, k/4) particles) to log(h / s), s being the side of
the adaptive cell.  Its only use is the first search radius and the first h guess
of the neighbour search; the converged neighbours and h are exactly those of
the plain method, so a bad prediction costs time, never accuracy.

Inference, training (forward + backward) and the Adam update all run in this
project's CUDA kernels (mg_seed_features, mg_mlp_forward, mg_mlp_train_step);
PyTorch only holds the buffers.
"""
from __future__ import annotations

import math
import os

import numpy as np
import torch

from . import _native as N
from ._native import check, ptr

__all__ = ["SeedModel", "resolve_model", "train_seed_model", "default_model_path"]

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
P = N.MG_MLP_PARAM_COUNT
IN, HID = N.MG_MLP_IN_PAD, N.MG_MLP_HIDDEN
OFF_W1, OFF_B1 = 0, HID * IN
OFF_W2, OFF_B2 = OFF_B1 + HID, OFF_B1 + HID + HID * HID
OFF_W3, OFF_B3 = OFF_B2 + HID, OFF_B2 + 2 * HID


def default_model_path(k: int = 32) -> str:
    return os.path.join(_DATA, f"seed_mlp_k{k}.npz")


def _stream():
    import ctypes
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _bf16_bits(t: torch.Tensor) -> torch.Tensor:
    return t.to(torch.bfloat16).view(torch.int16).contiguous()


class SeedModel:
    def __init__(self, params: torch.Tensor, radius_factor: float = 1.15, meta=None):
        self.params = params.float().contiguous()
        self.device = params.device
        self.radius_factor = float(radius_factor)
        self.meta = dict(meta or {})
        self.refresh()

    # -- weights
    def refresh(self):
        p = self.params
        self.w1 = _bf16_bits(p[OFF_W1:OFF_B1])
        self.w2 = _bf16_bits(p[OFF_W2:OFF_B2])
        self.w3 = _bf16_bits(p[OFF_W3:OFF_B3])
        self.b1 = p[OFF_B1:OFF_W2]
        self.b2 = p[OFF_B2:OFF_W3]
        self.b3 = p[OFF_B3:OFF_B3 + 1]

    @classmethod
    def init(cls, device, seed: int = 0, bias: float = 0.0):
        g = torch.Generator().manual_seed(seed)
        p = torch.zeros(P)
        w1 = torch.randn(HID, IN, generator=g) * math.sqrt(2.0 / N.MG_MLP_IN)
        w1[:, N.MG_MLP_IN:] = 0.0
        p[OFF_W1:OFF_B1] = w1.flatten()
        p[OFF_W2:OFF_B2] = (torch.randn(HID, HID, generator=g) * math.sqrt(2.0 / HID)).flatten()
        p[OFF_W3:OFF_B3] = torch.randn(HID, generator=g) * math.sqrt(1.0 / HID)
        p[OFF_B3] = bias
        return cls(p.to(device))

    def save(self, path: str):
        os.makedirs(os.path.dirname(path), exist_ok=True)
        np.savez(path, params=self.params.cpu().numpy(), radius_factor=self.radius_factor,
                 **{f"meta_{k}": v for k, v in self.meta.items()})

    @classmethod
    def load(cls, path: str, device):
        with np.load(path) as z:
            meta = {k[5:]: z[k].item() if z[k].ndim == 0 else z[k] for k in z.files if k.startswith("meta_")}
            return cls(torch.as_tensor(z["params"], device=device), float(z["radius_factor"]), meta)

    # -- inference
    def features(self, cells, queries, nq, k):
        lib = N.load()
        feat = torch.empty((nq, IN), dtype=torch.int16, device=self.device)
        side = torch.empty(nq, dtype=torch.float32, device=self.device)
        check(lib.mg_seed_features(cells, ptr(queries), nq, k, ptr(feat), ptr(side), _stream()), "mg_seed_features")
        return feat, side

    def forward(self, feat, side=None):
        lib = N.load()
        n = feat.shape[0]
        out = torch.empty(n, dtype=torch.float32, device=self.device)
        seed = torch.empty(n, dtype=torch.float32, device=self.device) if side is not None else None
        check(lib.mg_mlp_forward(ptr(feat), n, ptr(self.w1), ptr(self.b1), ptr(self.w2), ptr(self.b2), ptr(self.w3),
                                 ptr(self.b3), ptr(side), ptr(out), ptr(seed), _stream()), "mg_mlp_forward")
        return out, seed

    def predict(self, cells, queries, nq, k):
        feat, side = self.features(cells, queries, nq, k)
        _, seed = self.forward(feat, side)
        return seed


_cache = {}


def resolve_model(seed, device, k: int = 32) -> SeedModel:
    if isinstance(seed, SeedModel):
        return seed
    if seed == "learned":
        path = default_model_path(k)
        key = (path, str(device))
        if key not in _cache:
            if not os.path.exists(path):
                raise FileNotFoundError(f"no trained seed network at {path}; train one with "
                                        "meshoid_gb300.seed_model.train_seed_model")
            _cache[key] = SeedModel.load(path, device)
        return _cache[key]
    if isinstance(seed, str) and os.path.exists(seed):
        return SeedModel.load(seed, device)
    raise ValueError(f"unknown seed {seed!r}")


def training_pairs(meshoid, model: SeedModel):
    """(features, log(h / s), s, k-th neighbour distance) for every query of a solved Meshoid."""
    m = meshoid
    feat, side = model.features(m._cells, m._queries, m.Nmask, m.des_ngb)
    # per-query h in the internal (slot) order the features are in
    h = m._hsml_q
    target = torch.log(h / side)
    return feat, target, side


def train_seed_model(snapshots, k: int = 32, steps: int = 3000, batch: int = 16384, lr: float = 2e-3,
                     seed: int = 0, device=None, quantile: float = 0.97, log=None) -> SeedModel:
    """Train the seed network on solved snapshots (Meshoid objects built with the
    plain seed).  Targets are the plain solver's converged h.  The returned
    model's radius_factor is the given quantile of r_k / h_pred on the training
    data (r_k = distance to the k-th neighbour), so about 1 - quantile of the
    queries need a second search pass."""
    device = device or snapshots[0].device
    lib = N.load()
    feats, targets, rks, hs = [], [], [], []
    probe = SeedModel.init(device, seed)
    for m in snapshots:
        f, t, s = training_pairs(m, probe)
        feats.append(f)
        targets.append(t)
        rks.append(m._kth_distance())
        hs.append(s)
    X = torch.cat(feats)
    Y = torch.cat(targets).float().contiguous()
    RK = torch.cat(rks)
    S = torch.cat(hs)
    model = SeedModel.init(device, seed, bias=float(Y.mean()))
    m_state = torch.zeros(P, device=device)
    v_state = torch.zeros(P, device=device)
    loss = torch.zeros(1, device=device)
    wsb = lib.mg_mlp_train_workspace_bytes(batch)
    ws = torch.empty(wsb, dtype=torch.uint8, device=device)
    gen = torch.Generator(device=device).manual_seed(seed)
    n = X.shape[0]
    history = []
    for step in range(1, steps + 1):
        idx = torch.randint(0, n, (batch,), device=device, generator=gen)
        xb = X[idx].contiguous()
        yb = Y[idx].contiguous()
        cur_lr = lr * 0.5 * (1.0 + math.cos(math.pi * step / steps))
        check(lib.mg_mlp_train_step(ptr(xb), ptr(yb), batch, ptr(model.params), ptr(m_state), ptr(v_state), step,
                                    float(cur_lr), ptr(model.w1), ptr(model.w2), ptr(model.w3), ptr(loss), None,
                                    ptr(ws), wsb, _stream()), "mg_mlp_train_step")
        if step % 250 == 0 or step == steps:
            history.append((step, float(loss)))
            if log:
                log(f"step {step}: batch mse {history[-1][1]:.5f}")
    model.refresh()
    out, pred = model.forward(X, S)
    ratio = (RK / pred.double()).float()
    model.radius_factor = float(torch.quantile(ratio[torch.randperm(ratio.numel(), device=device)[:1 << 20]],
                                               quantile))
    resid = (out - Y)
    model.meta = {"k": k, "steps": steps, "batch": batch, "n_train": int(n), "quantile": quantile,
                  "train_rmse_log": float(resid.pow(2).mean().sqrt()), "target_std": float(Y.std()),
                  "history": np.array(history)}
    return model
