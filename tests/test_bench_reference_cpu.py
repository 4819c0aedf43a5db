"""bench.py's reference arm on the host (no GPU): the JSON line keeps the
contract the GPU arm's line keeps (metric, unit, direction, the CPU
baseline it is, an end-to-end entry with no host-device copies), on a small
workload so that the test stays quick."""
import argparse
import io
import json
import sys
from contextlib import redirect_stdout
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def test_reference_arm_prints_one_contract_line(monkeypatch):
    import bench
    monkeypatch.setattr(bench, "IMAX", 256)
    monkeypatch.setattr(bench, "JMAX", 64)
    monkeypatch.setattr(bench, "NRECTS", 4)
    monkeypatch.setattr(bench, "CELLS", 256 * 64)
    monkeypatch.delenv("RANK", raising=False)
    args = argparse.Namespace(gpus=1, steps=2, warmup=1, ref_cap=3, ref_full_steps=1,
                              ref_parallel=1, arith="fast")
    out = io.StringIO()
    with redirect_stdout(out):
        bench.run_reference(args)
    lines = [l for l in out.getvalue().splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == "cell-updates/s"
    assert d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["steps"] == 2 and d["warmup"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert abs(d["value"] - bench.CELLS / (d["ms_per_step"] / 1e3)) <= 1e-6 * d["value"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == 1 and cb["value"] == d["value"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert d["config"]["solver"].startswith("lexicographic SOR")
    full = d["full_step"]
    assert len(full["ticks"]) == 2 and full["measured_full_step_ms"] > 0
    assert all(t["sor_iterations"] >= 1 for t in full["ticks"])
    # the extrapolation and the whole-tick measurement describe the same tick
    assert abs(full["model_error"]) < 0.5, full
    # the whole run: every tick, the model over the same iteration counts
    assert full["whole_run_sweeps"] == sum(t["sor_iterations"] for t in full["ticks"])
    assert abs(full["whole_run_s"] - sum(t["ms"] for t in full["ticks"]) / 1e3) < 1e-9
    assert abs(full["whole_run_model_s"] - full["whole_run_s"]) < 0.5 * full["whole_run_s"]
    import os
    if (os.cpu_count() or 1) > 1:
        par = d["cpu_all_cores_red_black"]
        assert par["threads"] == os.cpu_count() and par["value"] > 0


def test_reference_arm_prints_nothing_on_other_ranks(monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    out = io.StringIO()
    with redirect_stdout(out):
        bench.run_reference(argparse.Namespace(gpus=2, steps=1, warmup=1, ref_cap=1,
                                               ref_full_steps=1, ref_parallel=1,
                                               arith="fast"))
    assert out.getvalue() == ""


def test_launch_count_follows_the_solve_graph():
    """bench.py counts the kernels the FAST step graph launches from the
    length of the solve's WHILE body, which must be the library's
    kFastBodyIters."""
    import re
    from pathlib import Path
    import bench
    src = (Path(__file__).resolve().parent.parent / "stroemung_gb300" / "csrc" /
           "strm_kernels.cu").read_text()
    m = re.search(r"constexpr int kFastBodyIters = (\d+);", src)
    assert m and int(m.group(1)) == bench.FAST_BODY_ITERS
