"""Summaries of Nsight Compute output for profiles/.

  python -m kevernals_gb300.ncu_summary launches <launches.csv>
      per-kernel launch count, total time and share from an
      `ncu --metrics gpu__time_duration.sum --csv` launch list
  python -m kevernals_gb300.ncu_summary report <file.ncu-rep> [kernel-regex]
      the roofline / memory / stall metrics of the captured launches
      (reads the report with `ncu -i ... --page raw --csv`)
"""
from __future__ import annotations

import csv
import io
import re
import subprocess
import sys
from collections import OrderedDict

METRICS = [
    ("gpu__time_duration.sum", "duration"),
    ("dram__bytes_read.sum", "DRAM read"),
    ("dram__bytes_write.sum", "DRAM write"),
    ("gpu__dram_throughput.avg.pct_of_peak_sustained_elapsed", "DRAM throughput % of peak"),
    ("lts__t_sector_hit_rate.pct", "L2 hit rate %"),
    ("l1tex__t_sector_hit_rate.pct", "L1 hit rate %"),
    ("sm__throughput.avg.pct_of_peak_sustained_elapsed", "SM throughput %"),
    ("sm__inst_executed_pipe_lsu.avg.pct_of_peak_sustained_active", "LSU pipe %"),
    ("smsp__issue_active.avg.pct_of_peak_sustained_active", "issue active %"),
    ("sm__warps_active.avg.pct_of_peak_sustained_active", "achieved occupancy %"),
    ("smsp__thread_inst_executed_per_inst_executed.ratio", "threads per warp instruction"),
    ("smsp__inst_executed.sum", "warp instructions"),
    ("launch__registers_per_thread", "registers / thread"),
    ("launch__grid_size", "grid size"),
    ("launch__block_size", "block size"),
    ("sm__pipe_tensor_cycles_active.avg.pct_of_peak_sustained_active", "tensor pipe %"),
]
STALL_RE = re.compile(r"smsp__average_warps_issue_stalled_(\w+)_per_issue_active\.ratio")


def launches(path):
    rows = list(csv.DictReader(_skip_preamble(open(path))))
    per = OrderedDict()
    for r in rows:
        if r.get("Metric Name") != "gpu__time_duration.sum":
            continue
        name = r["Kernel Name"].split("(")[0]
        val = float(r["Metric Value"].replace(",", ""))
        unit = r.get("Metric Unit", "ns")
        scale = {"ns": 1e-6, "us": 1e-3, "usecond": 1e-3, "ms": 1.0, "msecond": 1.0,
                 "nsecond": 1e-6, "s": 1e3, "second": 1e3}.get(unit, 1e-6)
        n, t = per.get(name, (0, 0.0))
        per[name] = (n + 1, t + val * scale)
    total = sum(t for _, t in per.values())
    out = [f"{'kernel':60s} {'launches':>8s} {'total ms':>11s} {'share':>7s}"]
    for name, (n, t) in sorted(per.items(), key=lambda kv: -kv[1][1]):
        out.append(f"{name[:60]:60s} {n:8d} {t:11.3f} {100 * t / total:6.1f}%")
    out.append(f"{'total':60s} {sum(n for n, _ in per.values()):8d} {total:11.3f}")
    return "\n".join(out)


def _skip_preamble(f):
    lines = f.readlines()
    for i, line in enumerate(lines):
        if line.startswith('"ID"') or line.startswith("ID,"):
            return io.StringIO("".join(lines[i:]))
    return io.StringIO("".join(lines))


def report(path, kernel_regex=None):
    raw = subprocess.run(["ncu", "-i", path, "--page", "raw", "--csv"], capture_output=True,
                         text=True, check=True).stdout
    rows = list(csv.reader(io.StringIO(raw)))
    header, units, data = rows[0], rows[1], rows[2:]
    col = {h: i for i, h in enumerate(header)}
    out = []
    for r in data:
        kname = r[col["Kernel Name"]]
        if kernel_regex and not re.search(kernel_regex, kname):
            continue
        out.append(f"kernel: {kname[:150]}")
        for m, label in METRICS:
            if m in col:
                out.append(f"  {label:32s} {r[col[m]]:>18s} {units[col[m]]}")
        stalls = []
        for h, i in col.items():
            mm = STALL_RE.fullmatch(h)
            if mm:
                try:
                    stalls.append((float(r[i]), mm.group(1)))
                except ValueError:
                    pass
        stalls.sort(reverse=True)
        out.append("  top warp stall reasons (cycles per issued instruction):")
        for v, name in stalls[:8]:
            out.append(f"    {name:28s} {v:8.2f}")
    return "\n".join(out)


if __name__ == "__main__":
    if sys.argv[1] == "launches":
        print(launches(sys.argv[2]))
    else:
        print(report(sys.argv[2], sys.argv[3] if len(sys.argv) > 3 else None))
