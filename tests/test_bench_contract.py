"""bench.py's JSON contract on CPU: the committed headline line has every key
and a consistent roofline, the reference arm runs here and prints its line, and
the committed ncu tables hold what bench.py reads from them."""

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
KEYS = ["metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "gpu_launches", "roofline", "cpu_baseline", "e2e", "clocks"]


def test_committed_headline_line():
    d = json.loads((ROOT / "profiles" / "bench_serial-chain_65536.json").read_text())
    assert [k for k in KEYS if k not in d] == []
    assert d["config"]["workload"].startswith("serial-chain")
    r = d["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r
    assert abs(r["frac"] - r["achieved"] / r["peak"]) <= 1e-9 * r["frac"]
    assert 0.0 < r["frac"] < 1.5
    assert d["gpu_launches"] >= 1
    assert set(d["e2e"]) >= {"value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"}
    assert d["e2e"]["h2d_bytes_per_step"] > 0 and d["e2e"]["d2h_bytes_per_step"] > 0
    assert set(d["cpu_baseline"]) >= {"value", "unit", "cores", "kind", "sample"}
    assert d["clocks"]["reasons"] == [] or "sw_power_cap" in d["clocks"]["reasons"]
    # the headline is the fastest form within the q̈ bar (every instance within 1e-5)
    for name, m in d["modes"].items():
        err = m["qdd_rel_err_vs_fp64_crba"] or {}
        if all(e.get("bounded", e)["frac_le_1e-5"] == 1.0 for e in err.values()):
            assert m["value"] <= d["value"] * (1 + 1e-12), name


def test_configurations_default_to_their_own_batch_and_length(monkeypatch):
    """`bench.py --config k` runs configuration k's own batch and length: 1,024
    acrobots × 10,000 steps, 65,536 chains × 2,000 (the default run), 32,768
    cubes × 20,000, 16,384 quadrupeds × 10,000, each at its own dt."""
    sys.path.insert(0, str(ROOT))
    import bench

    want = {0: (1024, 10000, 1e-3), 1: (65536, 2000, 5e-4), 2: (32768, 20000, 1e-4), 3: (16384, 10000, 2e-4)}
    for k, (n, steps, dt) in want.items():
        monkeypatch.setattr(sys, "argv", ["bench.py", "--config", str(k)])
        a = bench.parse()
        assert (a.instances, a.steps, bench.DT[k]) == (n, steps, dt), k
    monkeypatch.setattr(sys, "argv", ["bench.py", "--gpus", "1", "--steps", "5", "--warmup", "3"])
    a = bench.parse()
    assert (a.config, a.instances, a.steps, a.warmup) == (1, 65536, 5, 3)


def test_committed_lines_record_their_mapping():
    """Every committed bench line records each form's launch shape; where the
    autotuner chose several lanes per instance, the line carries the one-lane
    run it was compared with and the chosen shape was the faster; the small
    batches of chains pick the body-parallel mapping."""
    sys.path.insert(0, str(ROOT))
    import bench

    picked = {}
    for f in sorted((ROOT / "profiles").glob("bench_*.json")):
        d = json.loads(f.read_text().strip().splitlines()[-1])
        if not d["config"]["workload"].split(" x ")[0] in bench.CONFIG_NAME.values():
            continue  # the cuboid-collider and velocity-stepping benchmarks have no mapping choice
        for name, m in d["modes"].items():
            launch = m["launch"]
            assert {"warps_per_sm", "coop_min_dof", "lanes_per_instance"} <= set(launch), (f.name, name)
            lanes = launch["lanes_per_instance"]
            assert lanes in (1, 2, 4, 8, 16, 32, 128), (f.name, name)
            if lanes > 1:
                assert m["value"] >= launch["one_lane"]["value"], (f.name, name)
                assert "body-parallel" in m["algorithm"], (f.name, name)
            picked[(f.name, name)] = lanes
        assert d.get("kernel_source_sha16") == bench.kernel_source_hash(), f.name
    assert picked[("bench_serial-chain_1024.json", "fp64_crba")] > 1
    assert picked[("bench_serial-chain_256.json", "fp64_crba")] > 1
    assert picked[("bench_serial-chain_65536.json", "mixed")] == 1


def test_ncu_tables_hold_what_bench_reads():
    t = json.loads((ROOT / "profiles" / "dram_traffic_per_instance_step.json").read_text())
    m = t["serial-chain"]["mixed"]
    assert m["dram_bytes_per_instance_step"] > 0 and m["warp_instructions_per_instance_step"] > 0
    assert "capture" in m
    # captured on the kernel sources in the tree (bench.py ignores a table of other sources)
    sys.path.insert(0, str(ROOT))
    import bench

    assert m["source_sha16"] == bench.kernel_source_hash()
    v = json.loads((ROOT / "profiles" / "vstep_work.json").read_text())
    assert v["fp64_flops_per_instance_step"] > 0 and "source" in v
    c = json.loads((ROOT / "profiles" / "collision_work.json").read_text())
    assert c["gripper"]["mean_flops_per_evaluation"] > 0


def test_reference_arm_prints_its_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "higher_is_better", "config", "cpu_baseline", "e2e"):
        assert k in line
    assert line["value"] > 0 and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def test_reference_arm_loads_no_cuda_library():
    """The reference arm builds its inputs with the CPU build of the workload
    generator: running it maps neither libgpb.so nor the CUDA runtime."""
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '1', "
            "'--instances', '512']; import bench; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "print('MAPS', 'libgpb.so' in maps, 'libcudart' in maps)")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip().splitlines()[-1] == "MAPS False False"


def test_oracle_workload_generator_matches_the_library():
    """oracle.from_config (CPU build) and gpb.Model.from_config (libgpb.so) give
    identical tables and initial states for every configuration."""
    import numpy as np

    import oracle
    from gpb import Model

    for config in range(4):
        A = Model.from_config(config, 300, seed=11)
        B = oracle.from_config(config, 300, seed=11)
        for x, y in zip(A[1:], B[1:]):
            np.testing.assert_array_equal(x, y)
        for name in Model.FIELDS:
            np.testing.assert_array_equal(getattr(A[0], name), getattr(B[0], name), err_msg=name)
