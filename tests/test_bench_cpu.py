"""bench.py's reference arm, which runs on the host cores only: the JSON line
it prints carries the keys of the benchmark contract, rank 0 alone prints
under a multi-rank launch, and the workloads that time the reference inside
their own line say so and exit cleanly."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench(*args, env=None, timeout=300):
    e = dict(os.environ)
    e.update(env or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                       timeout=timeout, cwd=ROOT, env=e)
    assert r.returncode == 0, r.stdout + r.stderr
    return [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]


def _oracle_built():
    try:
        from oracle import oracle as O
        O.num_threads()
    except Exception:  # noqa: BLE001 -- any failure means the oracle library is not there
        return False
    return True


def test_reference_arm_line_has_the_contract_keys():
    if not _oracle_built():
        pytest.skip("oracle library not built")
    lines = _bench("--impl", "reference", "--workload", "c0", "--steps", "2", "--warmup", "1")
    assert len(lines) == 1
    d = lines[0]
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 1
    assert d["value"] > 0 and d["unit"] == "queries/s" and d["higher_is_better"] is True
    assert "workload" in d["config"]
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_prints_on_rank_zero_only():
    lines = _bench("--impl", "reference", "--workload", "c0", "--steps", "1", "--warmup", "1",
                   env={"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert lines == []


@pytest.mark.parametrize("workload", ["c4", "bf", "latency"])
def test_reference_arm_of_self_timed_workloads(workload):
    lines = _bench("--impl", "reference", "--workload", workload)
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and "unavailable" in lines[0]
