"""Train the seed network on generated snapshots (GPU, this project's kernels).

    python -m meshoid_gb300.train_seed --n 4194304 --snapshots 8 --dist plummer \\
        --out meshoid_gb300/data/seed_mlp_k32.npz

Each snapshot is solved with the plain seed; its converged h are the targets.
The plain seed's radius factor is calibrated on the same snapshots (the same
quantile of r_k / h_seed), so the learned and plain seeds are compared at the
same expected re-search rate.
"""
from __future__ import annotations

import argparse
import time

import numpy as np
import torch

from . import synthetic
from .meshoid import Meshoid
from .seed_model import default_model_path, train_seed_model


def make_snapshot(dist: str, n: int, seed: int) -> np.ndarray:
    if dist == "plummer":
        return synthetic.plummer(n, seed=seed)
    if dist == "clumps":
        return synthetic.clump_mixture(n, seed=seed)
    if dist == "uniform":
        return synthetic.uniform(n, seed=seed)
    raise ValueError(dist)


def plain_radius_factor(snapshots, quantile: float) -> float:
    """Quantile of r_k / h_plain over the snapshots' queries."""
    import ctypes

    from . import _native as N
    ratios = []
    for m in snapshots:
        seed = torch.empty(m.Nmask, dtype=torch.float32, device=m.device)
        N.check(N.load().mg_seed_plain(m._cells, N.ptr(m._queries), m.Nmask, m.des_ngb, N.ptr(seed),
                                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "mg_seed_plain")
        ratios.append((m._kth_distance() / seed.double()).float())
    r = torch.cat(ratios)
    sub = r[torch.randperm(r.numel(), device=r.device)[:1 << 20]]
    return float(torch.quantile(sub, quantile))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1 << 22)
    ap.add_argument("--snapshots", type=int, default=8)
    ap.add_argument("--dist", default="plummer", help="comma list: plummer, clumps, uniform")
    ap.add_argument("--k", type=int, default=32)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--quantile", type=float, default=0.97)
    ap.add_argument("--seed0", type=int, default=1000)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    dists = a.dist.split(",")
    t0 = time.time()
    snaps = []
    for i in range(a.snapshots):
        d = dists[i % len(dists)]
        pos = make_snapshot(d, a.n, a.seed0 + i)
        snaps.append(Meshoid(pos, des_ngb=a.k, seed="plain", radius_factor=1.6))
        print(f"snapshot {i} ({d}, {a.n}) solved")
    rf_plain = plain_radius_factor(snaps, a.quantile)
    model = train_seed_model(snaps, k=a.k, steps=a.steps, batch=a.batch, lr=a.lr, quantile=a.quantile,
                             log=print)
    model.meta.update({"dist": a.dist, "n_per_snapshot": a.n, "snapshots": a.snapshots,
                       "plain_radius_factor": rf_plain, "seed0": a.seed0})
    out = a.out or default_model_path(a.k)
    model.save(out)
    print(f"saved {out}: radius_factor {model.radius_factor:.4f} (plain {rf_plain:.4f}), "
          f"train rmse(log h) {model.meta['train_rmse_log']:.4f}, {time.time() - t0:.1f} s")


if __name__ == "__main__":
    main()
