"""bench.py's reference arm runs on the host cores only. It times the
reference 3D program's own statements, translated to C (oracle/_ref), or
the FP64 C++ restatement where that C is absent or --reference-port asks
for it. Its JSON line keeps the benchmark contract's keys in both forms,
checked here on short samples. The workloads whose CPU figure lives inside
their own line print one `unavailable` line and exit 0. No GPU work."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def bench_line(*args):
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    out = subprocess.run([sys.executable, "bench.py", *args], cwd=ROOT, env=env, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    return json.loads(lines[0])


def check_contract(d, kind):
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["metric"] == d["unit"] == "Mcell-updates/s" and d["steps"] == 1 and d["n_gpus"] == 1
    assert d["config"]["workload"] == "3d_plain_276cube" and d["config"]["grid"] == [276, 276, 276]
    cb = d["cpu_baseline"]
    assert cb["kind"] == kind and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "note" not in d, d.get("note")


def test_reference_arm_port_line_keeps_the_contract():
    d = bench_line("--impl", "reference", "--steps", "1", "--warmup", "0", "--cpu-sample-steps", "1",
                   "--reference-port")
    check_contract(d, "port")


def test_reference_arm_times_the_translated_reference_program():
    sys.path.insert(0, ROOT)
    from oracle import ref_f90c
    if not ref_f90c.translated_exists(ref_f90c.BENCH_TAG):
        pytest.skip("no translated reference program in oracle/_ref (built from the reference sources)")
    d = bench_line("--impl", "reference", "--steps", "1", "--warmup", "0")
    check_contract(d, "reference")
    assert d["cpu_baseline"]["cores"] == ref_f90c.PLAIN_3D_RANKS
    assert d["config"]["nstep_per_bench_step"] == ref_f90c.BENCH_SAMPLE_STEPS


@pytest.mark.parametrize("workload", ["2d_plain", "batch2d", "surrogate", "3d_large"])
def test_reference_arm_prints_unavailable_for_other_workloads(workload):
    d = bench_line("--impl", "reference", "--workload", workload)
    assert d["impl"] == "reference" and isinstance(d["unavailable"], str) and d["unavailable"]


def test_cpu_baseline_sample_is_sized_by_time():
    """The GPU line's cpu_baseline helper: without a step count it times as
    many steps as take about target_s (at least 2, at most max_steps); with
    one it times exactly that many."""
    sys.path.insert(0, ROOT)
    import bench
    from seismic_cpml_gb300 import params as P
    p, _ = P.small_3d(n=(40, 36, 32), nstep=500)
    v, dt, n = bench.cpu_baseline(p, 2, target_s=0.3, max_steps=300)
    assert 2 <= n <= 300 and dt > 0 and v > 0
    assert dt < 3.0                       # about target_s, not the cap
    v2, dt2, n2 = bench.cpu_baseline(p, 1, sample_steps=3)
    assert n2 == 3 and v2 > 0
