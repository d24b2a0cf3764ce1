"""bench.py's reference arm keeps the one-JSON-line contract on the CPU (it times the reference's CPU
algorithm, the oracle port, on the host cores and needs no GPU): rank 0 prints one line with the
metric, the throughput, the workload, the CPU-baseline description and an e2e entry with no host
copies; any other rank exits 0 without work."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(env_extra, *args):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_one_contract_line():
    r = run_bench({}, "--impl", "reference", "--steps", "2", "--warmup", "3")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["metric"] == "site-steps/s FP64"
    assert out["unit"] == "site-steps/s" and out["higher_is_better"] is True
    assert out["steps"] == 2 and out["warmup"] >= 3 and out["n_gpus"] == 1 and out["dtype"] == "f64"
    assert out["value"] > 0 and len(out["per_step_values"]) == 2
    cfg = out["config"]
    assert cfg["workload"].startswith("DNKG N=128") and cfg["chain_length"] == 128 and cfg["copies"] == 65536
    sample = cfg["sample_copies_per_step"]
    # the throughput is the sample's site-steps over the timed wall clock
    expect = cfg["chain_length"] * sample * cfg["kernel_batching"] / (out["ms_per_step"] * 1e-3)
    assert abs(out["value"] - expect) <= 1e-6 * expect
    cb = out["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == out["value"] and cb["sample"]
    assert out["e2e"] == {"value": out["value"], "unit": "site-steps/s", "h2d_bytes_per_step": 0,
                          "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_without_work():
    r = run_bench({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, "--impl", "reference", "--steps", "2",
                  "--warmup", "3")
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
