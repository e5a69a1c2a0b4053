"""bench.py's reference arm (the oracle port on the host cores; no GPU): one
JSON line with the keys the benchmark contract names."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["steps"] == 1 and line["warmup"] >= 3
    assert line["higher_is_better"] is True
    assert line["config"]["size"] == 1026 and line["config"]["gs_iterations"] == 20
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]


def test_summary_digest_of_a_bench_line():
    import bench
    line = {"value": 3.2e8, "e2e": {"value": 3.0e8},
            "roofline": {"frame_roofline_frac": 0.012, "alone_ms": 0.5, "latency_bound_ms": 0.08},
            "parity": {"status": "bit-exact"},
            "forms": {"batched": {"value": 1.1e9, "vs_plain": 3.4, "roofline": {"frac": 0.03}},
                      "precision": {"f16": {"value": 2e8, "vs_plain": 0.6}},
                      "differentiation": {"error": "RuntimeError: x"},
                      "fma": {"value": 3.3e8, "vs_plain": 1.03,
                              "rel_l2_vs_bit_exact_frame_1": {"density": 2e-7, "vx": 1e-7}}}}
    s = bench.summarize(line)
    assert s["plain"] == {"value": 3.2e8, "e2e": 3.0e8, "frame_frac": 0.012, "parity": "bit-exact",
                          "solve_alone_ms": 0.5, "latency_bound_ms": 0.08}
    assert s["fma"] == {"value": 3.3e8, "vs_plain": 1.03, "err": 2e-7, "error": None}
    assert s["batched"]["vs_plain"] == 3.4 and s["batched"]["frac"] == 0.03
    assert s["precision_f16"] == {"value": 2e8, "vs_plain": 0.6, "density_err_frame_1": None}
    assert s["differentiation"]["error"] == "RuntimeError: x"


def test_latency_bound_formula():
    import bench
    b = bench.latency_bound_ms(2000.0, strips=34, groups=4)
    chain = (2 * 1026 + 3 * 20) * 6 * 4 / 2.0e6  # ms at 2 GHz
    assert abs(b["chain_ms"] - chain) < 1e-12
    assert abs(b["handoff_ms"] - 36 * 1.5e-3) < 1e-12
    assert abs(b["latency_bound_ms"] - (chain + 0.054)) < 1e-12
