"""The ncu summary tool behind the committed profile summaries, on synthetic
ncu CSV output (no GPU, no report file)."""
import subprocess

from kevernals_gb300 import ncu_summary

HEADER = ('"ID","Process ID","Process Name","Host Name","Kernel Name","Context","Stream","Block Size",'
          '"Grid Size","Device","CC","Section Name","Metric Name","Metric Unit","Metric Value"\n')


def _row(i, kernel, unit, value, metric="gpu__time_duration.sum"):
    return (f'"{i}","1","python3","127.0.0.1","{kernel}(int, float *)","1","7","(32, 4, 1)","(64, 1, 1)",'
            f'"0","10.3","Command line profiler metrics","{metric}","{unit}","{value}"\n')


def test_launch_list_shares(tmp_path):
    csv_path = tmp_path / "launches.csv"
    csv_path.write_text("==PROF== Connected to process 1\n==PROF== Disconnected from process 1\n" + HEADER +
                        _row(0, "fwd", "ns", "3,000,000") + _row(1, "back", "us", "1000") +
                        _row(2, "fwd", "ms", "3") + _row(3, "fwd", "ns", "5", metric="dram__bytes_read.sum"))
    text = ncu_summary.launches(str(csv_path)).splitlines()
    rows = {ln.split()[0]: ln.split()[1:] for ln in text[1:]}
    assert rows["fwd"][:2] == ["2", "6.000"] and rows["fwd"][2] == "85.7%"
    assert rows["back"][:2] == ["1", "1.000"] and rows["back"][2] == "14.3%"
    assert rows["total"] == ["3", "7.000"]
    assert text[1].startswith("fwd")          # sorted by total time


def test_report_picks_metrics_and_stalls(monkeypatch):
    header = ["ID", "Kernel Name", "gpu__time_duration.sum", "dram__bytes_read.sum",
              "smsp__average_warps_issue_stalled_long_scoreboard_per_issue_active.ratio",
              "smsp__average_warps_issue_stalled_wait_per_issue_active.ratio"]
    units = ["", "", "ms", "byte", "ratio", "ratio"]
    data = [["0", "exact_fwd_kernel", "11.09", "1000", "5.91", "1.81"],
            ["1", "exact_back_kernel", "8.41", "2000", "4.69", "1.72"]]
    raw = "\n".join(",".join(f'"{c}"' for c in r) for r in [header, units] + data) + "\n"

    def fake_run(cmd, **kw):
        assert cmd[:2] == ["ncu", "-i"]
        return subprocess.CompletedProcess(cmd, 0, stdout=raw, stderr="")
    monkeypatch.setattr(ncu_summary.subprocess, "run", fake_run)
    text = ncu_summary.report("x.ncu-rep", "fwd")
    assert "exact_fwd_kernel" in text and "exact_back_kernel" not in text
    assert "11.09 ms" in text and "DRAM read" in text
    lines = text.splitlines()
    i = lines.index("  top warp stall reasons (cycles per issued instruction):")
    assert lines[i + 1].split() == ["long_scoreboard", "5.91"] and lines[i + 2].split() == ["wait", "1.81"]
