#!/usr/bin/env python
"""Benchmark: particles/s for smoothing lengths + first-order gradients.

Workload (one "step"): a Plummer sphere of N = 2^22 particles (a = 1, radii
truncated at 20a, isotropic directions, equal masses, seeded), des_ngb = 32:
build the cell index, seed h, find the 32 nearest neighbours and solve h,
then the first-order least-squares gradient of 5 field components (log
density, x*y*z, and the 3 components of a solid-body rotation plus N(0, 0.1)
noise) -- the drop-in equivalent of ``Meshoid(pos, m, des_ngb=32)`` followed
by ``M.D(f)``.  Inputs (positions, fields: 268 MB) exceed the 126 MB L2.

`value` is the throughput of the faster of the two h seeds (plain cell-count
seed, learned network seed) with inputs resident in HBM; both are reported
under "seeds".  "targets" adds the 2^24 clump mixture with F = 19 field
components (GPU vs the CPU path on a 2^20 sample), the 64-snapshot batch in
one CUDA graph, and the 3-D deposit and the ray tracer on the 2^22 Plummer
sphere (GPU vs the oracle's serial loops on a sample).  `e2e` is the same metric through
the public API with host (pinned) arrays: host->device copies of positions,
masses and fields and device->host copies of h and the gradients are inside
the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

N > 1 runs under torchrun as independent replicas (one per GPU, no
collectives on the data path; the per-step time is the max over ranks).
`--impl reference` times the CPU path (scipy cKDTree + the C/OpenMP
restatement of the reference loops) on the host cores.
"""
from __future__ import annotations

import argparse
import atexit
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "particles/s for hsml+gradient on 1 GB300, learned vs plain h-seed at 1e-6 h tol"
UNIT = "particles/s"
N_DEFAULT = 1 << 22
K = 32


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--cpu-sample", type=int, default=1 << 22,
                    help="particles of the CPU baseline timed beside the GPU run (default: the whole workload)")
    ap.add_argument("--ref-sample", type=int, default=N_DEFAULT,
                    help="particles per step of --impl reference (default: the whole workload)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--order2-refine", action="store_true",
                    help="also time the 2^24 clump target's order-2 sweep with each order-2 method")
    ap.add_argument("--no-targets", action="store_true",
                    help="skip the 2^24 clump-mixture, 19-component target measurement")
    ap.add_argument("--profile-case", type=int, default=0, metavar="N",
                    help="run only the hot path on an N-particle Plummer set (setup + 2 steps; for ncu)")
    ap.add_argument("--kernels-case", type=int, default=0, metavar="N",
                    help="run every profiled kernel once at size N (learned-seed search, D, D2, maps) and exit")
    ap.add_argument("--maps-case", type=int, default=0, metavar="N",
                    help="run only DepositToGrid (128^3) and radtransfer (1024^2, 3 bands) twice on an "
                         "N-particle Plummer set (for ncu)")
    return ap.parse_args()


def profile_case(n: int) -> int:
    """One setup solve and two timed-path steps (Meshoid + D of 5 components) at
    size n, nothing else: the command profiled under ncu."""
    import torch

    import meshoid_gb300
    pos, m, v = workload(n, seed=2)
    pd = torch.as_tensor(pos, device="cuda")
    md = torch.as_tensor(m, device="cuda")
    M = meshoid_gb300.Meshoid(pd, md, des_ngb=K)
    f = torch.cat([torch.log(M.density)[:, None], (pd[:, 0] * pd[:, 1] * pd[:, 2])[:, None],
                   torch.as_tensor(v, device="cuda")], 1).contiguous()
    for _ in range(2):
        M = meshoid_gb300.Meshoid(pd, md, des_ngb=K)
        d = M.D(f)
    torch.cuda.synchronize()
    print(f"profile case n={n} ok checksum={float(d.double().abs().sum()):.6e}")
    return 0


def kernels_case(n: int) -> int:
    """One pass over every kernel that has a per-kernel ncu summary, at size n
    (Plummer): cell index + learned seed + search + h, D of 5 components,
    D2 of the same fields (float-float), SurfaceDensity 1024^2,
    DepositToGrid 128^3, radtransfer 1024^2 x 3 bands: the command profiled
    under ncu, one kernel per capture."""
    import torch

    import meshoid_gb300
    from meshoid_gb300 import radiation, synthetic as S
    pos = S.plummer(n, seed=2)
    rng = np.random.default_rng(9)
    m = torch.as_tensor(rng.uniform(0.5, 1.5, n) / n, device="cuda")
    pt = torch.as_tensor(pos, device="cuda")
    M = meshoid_gb300.Meshoid(pt, m, des_ngb=K, seed="learned")
    f = torch.cat([torch.log(M.density)[:, None], (pt[:, 0] * pt[:, 1] * pt[:, 2])[:, None],
                   torch.as_tensor(S.rotation_velocity(pos, seed=3), device="cuda")], 1).contiguous()
    d1 = M.D(f)
    d2 = M.D2(f)
    sd = M.SurfaceDensity(m, center=[0.0, 0.0, 0.0], size=8.0, res=1024)
    g = M.DepositToGrid(m, size=8.0, center=[0.0, 0.0, 0.0], res=128)
    kappa = torch.as_tensor(rng.uniform(5e3, 5e4, (n, 3)), device="cuda")
    j = torch.as_tensor(rng.uniform(0.1, 2.0, (n, 3)), device="cuda")
    img = radiation.radtransfer(j, m, kappa, pt, M.kernel_radius, 1024, 8.0, [0.0, 0.0, 0.0])
    torch.cuda.synchronize()
    print(f"kernels case n={n} ok checksums {float(d1.abs().sum()):.6e} {float(d2.abs().sum()):.6e} "
          f"{float(sd.sum()):.6e} {float(g.sum()):.6e} {float(img.sum()):.6e}")
    return 0


def maps_case(n: int) -> int:
    """The two map targets of the bench (3-D deposit, ray tracer) at size n,
    twice each after the kNN set-up: the command profiled under ncu."""
    import torch

    import meshoid_gb300
    from meshoid_gb300 import radiation, synthetic as S
    pos = S.plummer(n, seed=2)
    rng = np.random.default_rng(9)
    m_t = torch.as_tensor(rng.uniform(0.5, 1.5, n) / n, device="cuda")
    pos_t = torch.as_tensor(pos, device="cuda")
    M = meshoid_gb300.Meshoid(pos_t, m_t, des_ngb=K)
    kappa = torch.as_tensor(rng.uniform(5e3, 5e4, (n, 3)), device="cuda")
    j = torch.as_tensor(rng.uniform(0.1, 2.0, (n, 3)), device="cuda")
    for _ in range(2):
        g = M.DepositToGrid(m_t, size=8.0, center=[0.0, 0.0, 0.0], res=128)
        img = radiation.radtransfer(j, m_t, kappa, pos_t, M.kernel_radius, 1024, 8.0, [0.0, 0.0, 0.0])
    torch.cuda.synchronize()
    print(f"maps case n={n} ok checksum={float(g.sum()):.6e} {float(img.sum()):.6e}")
    return 0


def max_over_ranks(ms: float, dist, device) -> float:
    """Per-step time of the job: the slowest rank's (replicas run the same
    workload each; with no process group, the value itself)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t)


def job_throughput(n_per_rank: int, world: int, ms: float) -> float:
    """Whole-job particles/s: every rank processes n_per_rank particles per step."""
    return n_per_rank * world / (ms * 1e-3)


def clumps_target(steps: int, cpu: bool, refine: bool = False):
    """The many-right-hand-side target: N = 2^24 clump mixture, 16 Fourier scalar
    fields + a 3-vector (F = 19), Meshoid + D order 1 per step; order 2 (D and
    D2 of the same fields, moments included) timed after one untimed call (with refine, also
    order2_with_refinement); the CPU path on a 2^20 sample of the same
    generator."""
    import torch

    import meshoid_gb300
    from meshoid_gb300 import synthetic as S
    n = 1 << 24
    pos = S.clump_mixture(n, seed=7)
    pos_t = torch.as_tensor(pos, device="cuda")
    m_t = torch.full((n,), 1.0 / n, dtype=torch.float64, device="cuda")
    f = torch.cat([S.fourier_fields_torch(pos_t, 16, seed=8), S.fourier_fields_torch(pos_t, 3, seed=9, kmax=8)], 1)
    f = f.contiguous()

    def step():
        M = meshoid_gb300.Meshoid(pos_t, m_t, des_ngb=K)
        return M, M.D(f)

    M, _ = step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        M, d = step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    # order 2: one untimed call (allocations), then two timed calls, each from
    # scratch (reset_dweights drops the cached moment factors, so every timed
    # call computes them again, as the first call of a new Meshoid does)
    d2 = M.D2(f)
    d1 = M.D(f, order=2)
    ms2 = 0.0
    for _ in range(2):
        M.reset_dweights()
        del d1, d2
        torch.cuda.synchronize()
        e0.record()
        d2 = M.D2(f)
        d1 = M.D(f, order=2)
        e1.record()
        torch.cuda.synchronize()
        ms2 += e0.elapsed_time(e1) / 2
    from meshoid_gb300 import _native as NAT
    out = {"workload": "clump mixture N=2^24 (64 clumps + 20% background), des_ngb=32, D order 1 of F=19 "
                       "(16 Fourier scalars + 3-vector)", "gpu_ms_per_step": ms, "gpu_value": n / (ms * 1e-3),
           "unit": UNIT, "order2_sweep_ms": ms2, "order2_method": "float-float",
           "order2_fp64_rows": (M._gstatus & NAT.MG_Q_FP64_SOLVE).ne(0).float().mean().item(),
           "fp64_band_rows": int(M.stats[3]), "heavy_queries": int(M.stats[9])}
    if refine:
        out.update(order2_methods(M, f))
    del M, d, d1, d2
    if cpu:
        ns = 1 << 20
        ps = S.clump_mixture(ns, seed=7)
        fs = np.c_[S.fourier_fields(ps, 16, seed=8), S.fourier_fields(ps, 3, seed=9, kmax=8)]
        t = cpu_pipeline(ps, None, fs)
        out["cpu_value"] = ns / t
        out["cpu_sample"] = f"clump mixture N={ns} (same generator), cKDTree + C/OpenMP HsmlIter + weights + D of 19, {t:.2f} s"
        out["speedup_vs_cpu"] = out["gpu_value"] / out["cpu_value"]
    torch.cuda.empty_cache()
    return out


def order2_methods(M, f):
    """The order-2 sweep (D2 and D order 2 of f) on M with each order-2 method:
    "float-float" (the default: float-float moments computed once per
    neighbour set and shared by both calls, FP64 re-solve of flagged rows),
    "fp32" (FP32 sweep, FP64 re-solve of flagged rows) and "fp32" with the
    refinement step; with the fraction of rows solved in FP64 and refined."""
    import torch

    import meshoid_gb300
    from meshoid_gb300 import _native as NAT
    out = {}
    for key, method, refine in (("float_float", "float-float", False), ("fp32", "fp32", False),
                                ("fp32_refined", "fp32", True)):
        prev_m = meshoid_gb300.set_order2_method(method)
        prev = meshoid_gb300.set_order2_refinement(refine)
        cthr = M.cond_threshold
        if method == "fp32":
            M.cond_threshold = (cthr[0], 1e5)
        try:
            M.reset_dweights()
            M._hsml_pair = None
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            M.D2(f)
            M.D(f, order=2)
            e1.record()
            torch.cuda.synchronize()
        finally:
            meshoid_gb300.set_order2_refinement(prev)
            meshoid_gb300.set_order2_method(prev_m)
            M.cond_threshold = cthr
        st = M._gstatus
        out[f"order2_{key}_ms"] = e0.elapsed_time(e1)
        out[f"order2_{key}_fp64_rows"] = (st & NAT.MG_Q_FP64_SOLVE).ne(0).float().mean().item()
        out[f"order2_{key}_refined_rows"] = (st & NAT.MG_Q_REFINED).ne(0).float().mean().item()
    return out


def maps_target(steps: int, cpu: bool):
    """The 3-D deposit (DepositToGrid, 128^3) and the ray tracer (radtransfer,
    1024^2, 3 bands) on the 2^22 Plummer sphere with its solved h; the CPU arm
    is the oracle's serial restatement of each (as the reference's own loops)
    on a bounded sample of the same particles."""
    import torch

    import meshoid_gb300
    from meshoid_gb300 import radiation, synthetic as S
    n = 1 << 22
    pos = S.plummer(n, seed=2)
    rng = np.random.default_rng(9)
    m = rng.uniform(0.5, 1.5, n) / n
    pos_t = torch.as_tensor(pos, device="cuda")
    m_t = torch.as_tensor(m, device="cuda")
    M = meshoid_gb300.Meshoid(pos_t, m_t, des_ngb=K)
    size, res = 8.0, 128
    kappa = torch.as_tensor(rng.uniform(5e3, 5e4, (n, 3)), device="cuda")
    j = torch.as_tensor(rng.uniform(0.1, 2.0, (n, 3)), device="cuda")
    ctr = [0.0, 0.0, 0.0]

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    ms_dep = timed(lambda: M.DepositToGrid(m_t, size=size, center=ctr, res=res))
    ms_rt = timed(lambda: radiation.radtransfer(j, m_t, kappa, pos_t, M.kernel_radius, 1024, size, ctr))
    out = {"deposit3d": {"workload": "DepositToGrid of m, 2^22 Plummer, 128^3 grid of side 8 a", "gpu_ms": ms_dep,
                         "gpu_value": n / (ms_dep * 1e-3), "unit": UNIT},
           "radtransfer": {"workload": "radtransfer, 2^22 Plummer, 1024^2 pixels of side 8 a, 3 bands",
                           "gpu_ms": ms_rt, "gpu_value": n / (ms_rt * 1e-3), "unit": UNIT}}
    if cpu:
        import time

        sys.path.insert(0, HERE)
        from oracle import oracle as O
        h = M.kernel_radius.cpu().numpy()
        hc = np.clip(h, size / (res - 1), 1e100)
        ns = 1 << 19
        t = time.perf_counter()
        O.grid_density(m[:ns], pos[:ns], hc[:ns], ctr, size, res, -1.0)
        t = time.perf_counter() - t
        out["deposit3d"].update({"cpu_value": ns / t, "cpu_sample": f"first {ns} particles, serial C restatement, "
                                                                   f"{t:.2f} s"})
        ns = 1 << 17
        t = time.perf_counter()
        O.radtransfer(j[:ns].cpu().numpy(), m[:ns], kappa[:ns].cpu().numpy(), pos[:ns], h[:ns], 1024, size, ctr, 0)
        t = time.perf_counter() - t
        out["radtransfer"].update({"cpu_value": ns / t, "cpu_sample": f"first {ns} particles, serial C restatement, "
                                                                     f"{t:.2f} s"})
        for v in out.values():
            v["speedup_vs_cpu"] = v["gpu_value"] / v["cpu_value"]
    del M
    torch.cuda.empty_cache()
    return out


def seed_target(steps: int):
    """The learned-seed workload: a Plummer sphere of 2^24 particles (density
    range ~1e6) on a seed the packaged network never saw (it was trained on
    seeds 1000-1007 at 2^22), neighbours and smoothing lengths at des_ngb 32
    with the plain seed and with the learned seed; per mode the seed and
    search stage times, the search's re-queued queries (mispredicted seeds),
    extra passes and candidates per query.  Both modes converge to the same
    neighbours and h (tests/test_gpu_seed.py).  Then the bound on any seed:
    the search given each particle's own k-th neighbour distance as its first
    guess (free and exact: what a perfect seed would predict) with a radius
    factor of 1.02, which covers every k-th neighbour with the margin the
    first pass's exactness test asks for."""
    import torch

    import meshoid_gb300
    from meshoid_gb300 import profiling
    from meshoid_gb300 import synthetic as S
    n = 1 << 24
    pos_t = torch.as_tensor(S.plummer(n, seed=2024), device="cuda")
    out = {"workload": "plummer N=2^24 (seed 2024, unseen in training), des_ngb=32: seed + neighbour search + h"}
    rec = profiling.StageRecorder()

    def timed(**kw):
        meshoid_gb300.Meshoid(pos_t, des_ngb=K, **kw)
        torch.cuda.synchronize()
        rec.reset()
        profiling.set_recorder(rec)
        for _ in range(steps):
            M = meshoid_gb300.Meshoid(pos_t, des_ngb=K, **kw)
        torch.cuda.synchronize()
        profiling.set_recorder(None)
        st = M.stats.cpu().numpy()
        stages = {k: v / steps for k, v in rec.totals().items()}
        return {"stages_ms": stages, "seed_plus_search_ms": stages.get("seed", 0.0) + stages.get("knn_hsml", 0.0),
                "mispredicted_seed_fraction": float(st[2]) / n, "extra_passes": int(st[0]),
                "candidates_per_query": float(st[1]) / n}

    for mode in ("plain", "learned"):
        out[mode] = timed(seed=mode)
    out["hsml_speedup_learned_vs_plain"] = out["plain"]["seed_plus_search_ms"] / out["learned"]["seed_plus_search_ms"]
    M0 = meshoid_gb300.Meshoid(pos_t, des_ngb=K)
    rk = torch.empty(n, dtype=torch.float32, device=pos_t.device)
    rk[M0._out_rows.long()] = M0._kth_distance().float()
    del M0
    b = timed(seed=rk, radius_factor=1.02)
    b["radius_factor"] = 1.02
    b["max_speedup_vs_plain"] = out["plain"]["seed_plus_search_ms"] / max(b["seed_plus_search_ms"], 1e-9)
    out["exact_rk_seed_bound"] = b
    torch.cuda.empty_cache()
    return out


def batched_target(steps: int):
    """Batched uneven snapshots: 64 snapshots, N log-uniform in [2^14, 2^21],
    each a Plummer sphere or a clump mixture by seed; per snapshot h, D order 1
    of 4 fields and a 1024^2 column density map; all of them in one CUDA graph
    (mg_batched_run) with cell parameters from the autotuner."""
    import torch

    from meshoid_gb300 import synthetic as S
    from meshoid_gb300.batch import SnapshotBatch, tune_cell_parameters
    rng = np.random.default_rng(5)
    sizes = np.exp(rng.uniform(np.log(2.0 ** 14), np.log(2.0 ** 21), 64)).astype(np.int64)
    snaps, kinds = [], []
    for i, n in enumerate(sizes):
        plummer = rng.random() < 0.5
        pos = S.plummer(int(n), seed=100 + i) if plummer else S.clump_mixture(int(n), seed=100 + i)
        pos_t = torch.as_tensor(pos, device="cuda")
        snaps.append((pos_t, None, S.fourier_fields_torch(pos_t, 4, seed=200 + i, kmax=8)))
        kinds.append("plummer" if plummer else "clumps")
    params = [tune_cell_parameters(sn[0], K) for sn in snaps]
    B = SnapshotBatch(snaps, des_ngb=K, map_res=1024, graph=True, cell_params=params).run()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(steps):
        B.launch()
    e1.record()
    B.run()
    ms = e0.elapsed_time(e1) / steps
    per = []
    for i, sn in enumerate(snaps):  # each snapshot alone (its own graph), for per-snapshot throughput
        b1 = SnapshotBatch([sn], des_ngb=K, map_res=1024, graph=True, cell_params=[params[i]]).run()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(3):
            b1.launch()
        e1.record()
        torch.cuda.synchronize()
        per.append(int(sizes[i]) / (e0.elapsed_time(e1) / 3 * 1e-3))
        del b1
    out = {"workload": "64 snapshots, N log-uniform in [2^14, 2^21], Plummer or clump mixture by seed; h, D order 1 "
                       "of 4 fields, 1024^2 SurfaceDensity each; one CUDA graph (mg_batched_run)",
           "particles": int(sizes.sum()), "ms_per_batch": ms, "value": float(sizes.sum()) / (ms * 1e-3), "unit": UNIT,
           "per_snapshot_particles_per_s": {"min": float(min(per)), "median": float(np.median(per)),
                                            "max": float(max(per))},
           "cell_params_chosen": sorted({str(p) for p in params}), "kinds": {k: kinds.count(k) for k in set(kinds)}}
    del B, snaps
    torch.cuda.empty_cache()
    return out


def bench_config(n: int, world: int = 1) -> dict:
    """The `config` object of both arms' JSON lines (the same workload)."""
    cfg = {"workload": f"plummer_2^{int(np.log2(n))}: Meshoid(pos, m, des_ngb=32) + D(f) of 5 components "
                       "(log rho, xyz, v_rot+noise)", "n_per_gpu": n, "des_ngb": K, "fields": 5,
           "parallelism": "replicas" if world > 1 else "single", "l2": "inputs (268 MB) exceed L2; no flush"}
    return cfg


def workload(n: int, seed: int):
    from meshoid_gb300 import synthetic as S
    pos = S.plummer(n, seed=seed)
    m = np.full(n, 1.0 / n)
    v = S.rotation_velocity(pos, omega=(0.0, 0.0, 1.0), sigma=0.1, seed=seed + 1)
    return pos, m, v


class ClockSampler:
    """nvidia-smi samples during the timed region (median SM clock, throttle reasons)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            atexit.register(self._end)  # no sampler outlives the bench, even after an error
        except Exception:
            self.proc = None

    def _end(self):
        if self.proc is not None and self.proc.poll() is None:
            self.proc.kill()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                pass

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, val in zip(names, p[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_pipeline(pos, m, fields, threads=None):
    """The reference path on the host: cKDTree (all cores) + the C restatement
    of HsmlIter / gradient_weights / D.  Returns seconds."""
    from scipy.spatial import cKDTree

    from oracle import oracle as O
    if threads:
        O.set_threads(threads)
    t0 = time.perf_counter()
    tree = cKDTree(pos)
    dist, ngb = O.knn(pos, K, tree=tree, workers=-1, extra=0)
    h, _ = O.hsml_iter(dist, dim=3, error_norm=1e-13)
    W, _ = O.gradient_weights(pos, ngb, h, np.arange(len(pos)), None, True, 1)
    O.apply_weights(W, ngb, np.arange(len(pos)), fields)
    return time.perf_counter() - t0


def cpu_fields(pos, m, v, h_rho=None):
    """log density comes from the solved density; the CPU path uses its own."""
    n = len(pos)
    lr = np.log(np.full(n, 1.0)) if h_rho is None else np.log(h_rho)
    return np.c_[lr, pos[:, 0] * pos[:, 1] * pos[:, 2], v]


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    from oracle import oracle as O
    O.build_oracle()
    cores = O.set_threads(cores)
    n = min(a.ref_sample, a.n)
    pos, m, v = workload(n, seed=2)
    f = cpu_fields(pos, m, v)
    for _ in range(max(a.warmup, 0)):
        cpu_pipeline(pos, m, f)
    times = [cpu_pipeline(pos, m, f) for _ in range(a.steps)]
    t = float(np.mean(times))
    val = n / t
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(n, int(os.environ.get("WORLD_SIZE", "1"))),
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"Plummer N={n} (same generator), full pipeline per step: cKDTree build+query"
                                       " (workers=-1) + C/OpenMP HsmlIter + gradient_weights + D"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    a = parse()
    if a.impl == "reference":
        return run_reference(a)
    if a.profile_case:
        return profile_case(a.profile_case)
    if a.maps_case:
        return maps_case(a.maps_case)
    if a.kernels_case:
        return kernels_case(a.kernels_case)
    import torch

    import meshoid_gb300
    from meshoid_gb300 import _native as N
    from meshoid_gb300 import profiling
    from meshoid_gb300.seed_model import default_model_path

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    lib = N.load()
    n = a.n
    pos, m, v = workload(n, seed=2 + rank)

    # resident inputs; log density from a setup solve (not timed)
    pos_d = torch.as_tensor(pos, device=dev)
    m_d = torch.as_tensor(m, device=dev)
    M0 = meshoid_gb300.Meshoid(pos_d, m_d, des_ngb=K)
    f_d = torch.stack([torch.log(M0.density), pos_d[:, 0] * pos_d[:, 1] * pos_d[:, 2]], 1)
    f_d = torch.cat([f_d, torch.as_tensor(v, device=dev)], 1).contiguous()
    del M0

    have_model = os.path.exists(default_model_path(K))
    if not have_model and rank == 0:
        print("# no packaged seed network: training one (not timed)", file=sys.stderr)
    if not have_model:
        from meshoid_gb300 import train_seed
        train_seed.main(["--n", str(min(n, 1 << 21)), "--snapshots", "4", "--steps", "1500"])

    def step(seed_mode):
        M = meshoid_gb300.Meshoid(pos_d, m_d, des_ngb=K, seed=seed_mode)
        d = M.D(f_d)
        return M, d

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    results = {}
    rec = profiling.StageRecorder()
    # clocks are sampled from the first warm-up to the end of the last timed
    # region, so that both seed modes' timed steps are covered
    sampler = ClockSampler(local)
    sampler.start()
    clocks = None
    for mode in ("plain", "learned"):
        for _ in range(max(a.warmup, 3)):
            step(mode)
        barrier()
        rec.reset()
        profiling.set_recorder(rec)
        l0 = lib.mg_launch_count()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        stats = None
        e0.record()
        for _ in range(a.steps):
            M, d = step(mode)
            stats = M.stats
        e1.record()
        barrier()
        profiling.set_recorder(None)
        launches = lib.mg_launch_count() - l0
        ms = max_over_ranks(e0.elapsed_time(e1) / a.steps, dist, dev)
        if mode == "learned":
            clocks = sampler.stop()
            clocks["window"] = "warm-up and timed steps of both seed modes"
        st = stats.cpu().numpy()
        results[mode] = {"ms": ms, "value": job_throughput(n, world, ms), "stages": {k: v / a.steps for k, v in
                                                                               rec.totals().items()},
                         "launches": launches // a.steps, "retries": int(st[2]), "extra_passes": int(st[0]),
                         "retries_first": int(M.first_pass_retries) if hasattr(M, "first_pass_retries") else int(st[2]),
                         "candidates_per_query": float(st[1]) / n, "newton_per_query": float(st[5]) / n,
                         "fp64_band": int(st[3])}

    # the headline is the faster seed mode (the same on every rank: the times
    # are already reduced over ranks); both are reported
    best = "learned" if results["learned"]["value"] > results["plain"]["value"] else "plain"

    # end to end through the public API with host buffers, with that seed
    pin_pos = torch.as_tensor(pos).pin_memory()
    pin_m = torch.as_tensor(m).pin_memory()
    f_host = f_d.cpu().pin_memory()
    h2d = pin_pos.numel() * 8 + pin_m.numel() * 8 + f_host.numel() * 8
    out_d = torch.empty((n, 5, 3), dtype=torch.float32).pin_memory()
    out_h = torch.empty(n, dtype=torch.float64).pin_memory()
    d2h = out_d.numel() * 4 + out_h.numel() * 8

    # Each step uploads its positions, masses and fields from pinned host
    # memory and reads back h and the gradients, as a caller streaming
    # snapshots would: the fields go up on a side stream while the search
    # runs, the results come back on another while the next step starts; the
    # timed region ends after the last read-back.
    h2d_stream = torch.cuda.Stream(device=dev)
    d2h_stream = torch.cuda.Stream(device=dev)

    def e2e_step():
        main = torch.cuda.current_stream()
        pos_d = pin_pos.to(dev, non_blocking=True)
        m_d = pin_m.to(dev, non_blocking=True)
        with torch.cuda.stream(h2d_stream):
            f_d = f_host.to(dev, non_blocking=True)
        M = meshoid_gb300.Meshoid(pos_d, m_d, des_ngb=K, seed=best)
        main.wait_stream(h2d_stream)
        f_d.record_stream(main)
        d = M.D(f_d)
        h = M.kernel_radius
        d2h_stream.wait_stream(main)
        with torch.cuda.stream(d2h_stream):
            out_d.copy_(d, non_blocking=True)
            out_h.copy_(h, non_blocking=True)
        d.record_stream(d2h_stream)
        h.record_stream(d2h_stream)

    for _ in range(max(a.warmup, 3)):
        e2e_step()
    torch.cuda.current_stream().wait_stream(d2h_stream)
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.steps):
        e2e_step()
    torch.cuda.current_stream().wait_stream(d2h_stream)
    e1.record()
    barrier()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1) / a.steps, dist, dev)

    if rank != 0:
        return 0
    other = "plain" if best == "learned" else "learned"
    L = results[best]
    P = results[other]
    # roofline of the dominant kernel stage (algorithmic bytes per particle)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    alg = {"knn_hsml": 12 + 4 * K + 4 + 4, "grad_sweep": 16 + 4 * K + 16 * 5}
    dom = max(alg, key=lambda s: L["stages"].get(s, 0.0))
    dom_ms = L["stages"][dom]
    achieved = n * alg[dom] / (dom_ms * 1e-3) / 1e9
    traffic = None
    try:
        tr = json.load(open(os.path.join(HERE, "profiles", "traffic.json")))
        traffic = tr.get(dom)
    except Exception:
        pass
    targets = None
    if not a.no_targets and world == 1:
        if not a.no_cpu_baseline:
            from oracle import oracle as O
            O.build_oracle()
            O.set_threads(os.cpu_count() or 1)
        targets = {"clumps_2^24_F19": clumps_target(3, cpu=not a.no_cpu_baseline, refine=a.order2_refine),
                   "learned_seed_2^24": seed_target(3),
                   "batched_64_snapshots": batched_target(3)}
        targets.update(maps_target(3, cpu=not a.no_cpu_baseline))
    cpu = None
    if not a.no_cpu_baseline and world == 1:
        from oracle import oracle as O
        O.build_oracle()
        cores = O.set_threads(os.cpu_count() or 1)
        ns = min(a.cpu_sample, n)
        ps, ms_, vs = workload(ns, seed=2)
        t = cpu_pipeline(ps, ms_, cpu_fields(ps, ms_, vs))
        cpu = {"value": ns / t, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"Plummer N={ns} (same generator), cKDTree build+query (workers=-1) + C/OpenMP HsmlIter"
                         f" + gradient_weights + D of 5 components, {t:.2f} s"}
    line = {
        "metric": METRIC, "value": L["value"], "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": max(a.warmup, 3), "ms_per_step": L["ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(n, world),
        "seed_mode": best,
        "seeds": {m: {"value": results[m]["value"], "ms_per_step": results[m]["ms"], "stages_ms": results[m]["stages"],
                      "retries": results[m]["retries"], "extra_passes": results[m]["extra_passes"],
                      "mispredicted_seed_fraction": results[m]["retries_first"] / n,
                      "candidates_per_query": results[m]["candidates_per_query"],
                      "newton_per_query": results[m]["newton_per_query"]} for m in ("plain", "learned")},
        "hsml_speedup_learned_vs_plain": (results["plain"]["stages"].get("seed", 0) +
                                          results["plain"]["stages"]["knn_hsml"]) /
                                         (results["learned"]["stages"].get("seed", 0) +
                                          results["learned"]["stages"]["knn_hsml"]),
        "e2e": {"value": job_throughput(n, world, e2e_ms), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms, "seed": best},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, "alg_bytes_per_particle": alg[dom],
                     "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"},
        "cpu_baseline": cpu,
        "targets": targets,
        "clocks": clocks,
        "gpu_launches": L["launches"] * a.steps,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
