"""Text summaries of ncu output for the kernels of this library.

    python -m meshoid_gb300.ncu_summary launches <ncu.csv>          # per-kernel launches, time, share
    python -m meshoid_gb300.ncu_summary traffic <ncu.csv> <calls> [scale]   # DRAM bytes per stage call
    python -m meshoid_gb300.ncu_summary report <file.ncu-rep>       # key counters of a --set full capture

The CSV input is what `ncu --metrics ... --csv --log-file <file>` writes.
"""
from __future__ import annotations

# Kernels of each C-ABI stage, for per-stage totals of an ncu launch list.
STAGE_KERNELS = {
    "build_cells": ("k_bbox", "k_frame", "k_keys", "k_radix", "k_slot_positions", "k_cell_count", "k_scan",
                    "k_brick"),
    "seed": ("k_seed_plain", "k_seed_features", "k_mlp_forward"),
    "knn_hsml": ("k_knn_group", "k_knn_hsml", "k_knn_heavy", "k_hsml_solve", "k_count_pass"),
    "load_fields": ("k_load_fields",),
    "grad_sweep": ("k_grad",),
}

_TIME = {"ns": 1e-6, "nsecond": 1e-6, "us": 1e-3, "usecond": 1e-3, "ms": 1.0, "msecond": 1.0}
_BYTES = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "KB": 1e3, "MB": 1e6, "GB": 1e9}


def _short(name: str) -> str:
    base = name.split("(")[0].replace("void ", "").strip()
    return base.split("::")[-1].split("<")[0] + ("<" + base.split("<", 1)[1] if "<" in base else "")


def read_ncu_csv(path: str):
    """Per-launch dicts {kernel, ms, dram_bytes} from `ncu --csv --log-file` output."""
    import csv
    with open(path) as fh:
        lines = [ln for ln in fh if not ln.startswith("==")]
    launches = {}
    for r in csv.DictReader(lines):
        key = r["ID"]
        d = launches.setdefault(key, {"kernel": _short(r.get("Kernel Name") or r.get("Function Name", "?")),
                                      "ms": 0.0, "dram_bytes": None})
        val = float(r["Metric Value"].replace(",", "") or 0)
        unit = r["Metric Unit"]
        if r["Metric Name"] == "gpu__time_duration.sum":
            d["ms"] = val * _TIME.get(unit, 1e-6)
        elif r["Metric Name"] in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
            d["dram_bytes"] = (d["dram_bytes"] or 0.0) + val * _BYTES.get(unit, 1.0)
    return list(launches.values())


def stage_of(kernel: str) -> str:
    for st, names in STAGE_KERNELS.items():
        if any(kernel.startswith(nm) for nm in names):
            return st
    return "other"


def summarize_launches(path: str) -> str:
    """Markdown table: per kernel its launches, total time and share (and DRAM
    bytes when the capture has them), then per-stage totals."""
    L = read_ncu_csv(path)
    agg = {}
    for d in L:
        a = agg.setdefault(d["kernel"], {"n": 0, "ms": 0.0, "bytes": 0.0, "has": False})
        a["n"] += 1
        a["ms"] += d["ms"]
        if d["dram_bytes"] is not None:
            a["bytes"] += d["dram_bytes"]
            a["has"] = True
    tot = sum(a["ms"] for a in agg.values()) or 1.0
    has_b = any(a["has"] for a in agg.values())
    out = ["| kernel | launches | total ms | share |" + (" DRAM MB |" if has_b else ""),
           "|---|---:|---:|---:|" + ("---:|" if has_b else "")]
    for k, a in sorted(agg.items(), key=lambda kv: -kv[1]["ms"]):
        out.append(f"| `{k[:60]}` | {a['n']} | {a['ms']:.3f} | {100 * a['ms'] / tot:.1f}% |" +
                   (f" {a['bytes'] / 1e6:.1f} |" if has_b else ""))
    out.append(f"| total | {sum(a['n'] for a in agg.values())} | {tot:.3f} | 100% |" + (" |" if has_b else ""))
    st = {}
    for k, a in agg.items():
        s = st.setdefault(stage_of(k), {"ms": 0.0, "bytes": 0.0})
        s["ms"] += a["ms"]
        s["bytes"] += a["bytes"]
    out += ["", "| stage | total ms | share |" + (" DRAM MB |" if has_b else ""),
            "|---|---:|---:|" + ("---:|" if has_b else "")]
    for k, s in sorted(st.items(), key=lambda kv: -kv[1]["ms"]):
        out.append(f"| {k} | {s['ms']:.3f} | {100 * s['ms'] / tot:.1f}% |" +
                   (f" {s['bytes'] / 1e6:.1f} |" if has_b else ""))
    return "\n".join(out)


def stage_traffic(path: str, calls: int, scale: float = 1.0) -> dict:
    """DRAM bytes per call of each stage (summed over its kernels, divided by
    the number of calls captured, times `scale` for a smaller captured case)."""
    tot = {}
    for d in read_ncu_csv(path):
        if d["dram_bytes"] is None:
            continue
        s = stage_of(d["kernel"])
        tot[s] = tot.get(s, 0.0) + d["dram_bytes"]
    return {k: v * scale / calls for k, v in tot.items()}


def summarize_report(rep: str) -> str:
    """Key counters of each launch in an `ncu --set full` report (ncu -i)."""
    import csv
    import subprocess
    out = subprocess.run(["ncu", "-i", rep, "--page", "raw", "--csv"], capture_output=True, text=True,
                         check=True).stdout
    rows = list(csv.reader(out.splitlines()))
    head, units = rows[0], rows[1]
    want = ["gpu__time_duration.sum", "dram__bytes_read.sum", "dram__bytes_write.sum",
            "gpu__dram_throughput.avg.pct_of_peak_sustained_elapsed", "sm__throughput.avg.pct_of_peak_sustained_elapsed",
            "sm__warps_active.avg.pct_of_peak_sustained_active", "smsp__issue_active.avg.pct_of_peak_sustained_active",
            "smsp__warps_eligible.avg.per_cycle_active", "l1tex__t_sector_hit_rate.pct", "lts__t_sector_hit_rate.pct",
            "launch__registers_per_thread", "launch__grid_size", "launch__block_size",
            "launch__occupancy_limit_registers", "launch__occupancy_limit_shared_mem",
            "smsp__thread_inst_executed_per_inst_executed.ratio", "sm__pipe_tensor_cycles_active.avg.pct_of_peak_sustained_active"]
    lines = []
    for r in rows[2:]:
        d = dict(zip(head, r))
        u = dict(zip(head, units))
        lines.append(f"### `{_short(d.get('Kernel Name', '?'))}`")
        for w in want:
            if w in d and d[w] != "":
                lines.append(f"- {w}: {d[w]} {u.get(w, '')}".rstrip())
        stalls = []
        for kk, v in d.items():
            if kk.startswith("smsp__average_warps_issue_stalled_") and kk.endswith("_per_issue_active.ratio") and v:
                try:
                    stalls.append((kk[len("smsp__average_warps_issue_stalled_"):-len("_per_issue_active.ratio")], float(v)))
                except ValueError:
                    pass
        stalls.sort(key=lambda x: -x[1])
        if stalls:
            lines.append("- top stall reasons (warps per issue): " +
                         ", ".join(f"{k} {v:.2f}" for k, v in stalls[:6]))
    return "\n".join(lines)


if __name__ == "__main__":
    import json
    import sys
    cmd = sys.argv[1] if len(sys.argv) > 1 else ""
    if cmd == "launches":
        print(summarize_launches(sys.argv[2]))
    elif cmd == "traffic":  # traffic <csv> <calls> [scale]
        print(json.dumps(stage_traffic(sys.argv[2], int(sys.argv[3]), float(sys.argv[4]) if len(sys.argv) > 4 else 1.0),
                         indent=1))
    elif cmd == "report":
        print(summarize_report(sys.argv[2]))
    else:
        print("usage: python -m meshoid_gb300.profiling launches <ncu.csv> | traffic <ncu.csv> <calls> [scale]"
              " | report <file.ncu-rep>")
        sys.exit(2)
