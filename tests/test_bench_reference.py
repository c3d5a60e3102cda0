"""The benchmark's reference arm runs on host cores only, so its JSON line
is checked here without a GPU: the reference's algorithm (the oracle's
all-pairs restatement of FluidSystemSPH::Run) timed on a bounded sample."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--workload", "plain_small", "--steps", "2",
           "--warmup", "1", "--ref-seconds", "0.3"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference"
    assert line["unit"] == "particle-steps/s" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["steps"] == 2 and line["warmup"] == 1 and line["vs_baseline"] is None
    assert line["config"]["workload"] == "plain_small" and line["config"]["particles"] == 16384
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == line["value"] and cb["cores"] >= 1
    assert cb["port_vs_reference"] > 0  # the port's speed against the reference's own Run
    # ms_per_step is the measured sample step, which fits in the run; the
    # whole-workload step is an extrapolation reported beside it
    assert line["ms_per_step"] * (line["steps"] + line["warmup"]) / 1e3 < 600
    assert line["ms_per_step_full_workload"] >= line["ms_per_step"]
    assert "extrapolated" in line["ms_per_step_full_workload_kind"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_gpus_flag_launches_ranks_dry_run():
    """--gpus 2 without a launcher starts two ranks itself (gloo here, no
    CUDA in the dry run); both join the barrier and rank 0 reports n_gpus 2,
    for either arm."""
    for impl in ("ours", "reference"):
        cmd = [sys.executable, "bench.py", "--gpus", "2", "--dry-run", "--impl", impl, "--steps", "1", "--warmup", "0"]
        env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
        r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
        assert r.returncode == 0, r.stderr[-2000:]
        lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
        assert len(lines) == 1, r.stdout
        assert lines[0]["n_gpus"] == 2 and lines[0]["dry_run"] and lines[0]["impl"] == impl
        assert lines[0]["max_over_ranks_s"] == 0.002  # rank 1's value: the max over ranks


def test_ncu_counters_ingest_and_match(tmp_path, monkeypatch):
    """Counters ingested from an ncu raw CSV are found again only for the
    same kernel, workload, kernel variant bits, cell size and kernel
    sources: the force pass ignores the density-only bits, the density pass
    does not."""
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setattr(bench, "COUNTERS", str(tmp_path / "counters.json"))
    raw = tmp_path / "raw.csv"
    names = ["Kernel Name", "dram__bytes_read.sum", "dram__bytes_write.sum", "smsp__inst_executed.sum",
             "gpu__time_duration.sum"]
    rows = [names, ["", "Mbyte", "Kbyte", "inst", "usecond"],
            ["void k_force<0, 4, 3, 1, 1>(DevArrays)", "400.5", "2,000", "1000", "500"],
            ["void k_force<0, 4, 3, 1, 1>(DevArrays)", "399.5", "1,000", "3000", "700"],
            ["void k_density<0, 0, 4, 1, 1, 1, 0, 1>(DevArrays)", "100", "10", "10", "400"]]
    raw.write_text("\n".join(",".join(f'"{c}"' for c in r) for r in rows) + "\n")
    v = 164088
    bench.ingest_ncu(str(raw), "plain_1m", v, 0.5, "cmd-f", "k_force")
    bench.ingest_ncu(str(raw), "plain_1m", v, 0.5, "cmd-d", "k_density")
    f, why = bench.ncu_counters("plain_1m", v, 0.5, "k_force")
    assert why is None and f["launches"] == 2 and f["command"] == "cmd-f"
    assert abs(f["dram_bytes"] - (400e6 + 1.5e6)) < 1 and f["warp_instructions"] == 2000
    assert abs(f["ncu_duration_s"] - 600e-6) < 1e-12
    d, why = bench.ncu_counters("plain_1m", v, 0.5, "k_density")
    assert why is None and d["launches"] == 1 and abs(d["dram_bytes"] - (100e6 + 10e3)) < 1
    # bit 64 selects density code only: the force entry still matches
    assert bench.ncu_counters("plain_1m", v & ~64, 0.5, "k_force")[0] is not None
    assert bench.ncu_counters("plain_1m", v & ~64, 0.5, "k_density")[0] is None
    assert bench.ncu_counters("plain_1m", v, 1.0, "k_force")[0] is None
    # counters of other kernel sources are not reported as the current kernels'
    monkeypatch.setattr(bench, "source_digest", lambda: "0" * 16)
    e, why = bench.ncu_counters("plain_1m", v, 0.5, "k_force")
    assert e is None and "other kernel sources" in why
