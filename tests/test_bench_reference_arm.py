"""bench.py --impl reference: the reference's CPU path (the oracle restatement
where the reference's sources are not built here) on a bounded sample of the
default workload, printed as one JSON line with the keys the benchmark
contract reads.  Runs on the CPU with a 4096-sample slice of the sample."""
import argparse
import json
import os
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line(monkeypatch, capsys, oracle_mod):
    sys.path.insert(0, REPO)
    import bench

    monkeypatch.setattr(bench, "CPU_NA", 1 << 12)
    args = argparse.Namespace(steps=1, warmup=0)
    bench.run_reference(args, 1, 0)
    lines = [l for l in capsys.readouterr().out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC
    assert line["unit"] == "comparisons/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["n_gpus"] == 1 and line["steps"] == 1 and line["warmup"] == 0
    assert line["config"]["workload"] == bench.SELF_WORKLOAD
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["unit"] == line["unit"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1
    assert "first 2^17 samples" in cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    # the rate is the sample's cells over the step time
    m = bench.SELF_M
    ns = (1 << 12) - m + 1
    e = m // 4
    cells = (ns - e) * (ns - e + 1) // 2
    assert abs(line["value"] - cells / (line["ms_per_step"] * 1e-3)) <= 1e-6 * line["value"]


def test_reference_arm_other_ranks_print_nothing(capsys):
    sys.path.insert(0, REPO)
    import bench

    bench.run_reference(argparse.Namespace(steps=1, warmup=0), 2, 1)
    assert capsys.readouterr().out == ""
