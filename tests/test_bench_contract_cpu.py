"""The benchmark's reference arm (the CPU restatement of the reference, timed
on the host cores) prints the JSON line the benchmark contract asks for, and
under torchrun only rank 0 runs it.  A 16^3 grid keeps it to a few seconds."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(env_extra):
    env = dict(os.environ, OMP_NUM_THREADS="2", **env_extra)
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--cells", "16", "--steps", "2",
                        "--warmup", "1"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return [ln for ln in r.stdout.splitlines() if ln.strip()]


@pytest.fixture(scope="module")
def ref_line(orc):  # the oracle library must exist (built by the fixture)
    lines = _run({})
    assert len(lines) == 1, lines
    return json.loads(lines[0])


def test_reference_arm_line_has_the_contract_keys(ref_line):
    d = ref_line
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["metric"] == "particle-pushes/s (full step, FP32)" and d["unit"] == "particle-pushes/s"
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["n_gpus"] == 1 and d["vs_baseline"] is None
    assert "16^3" in d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_runs_on_rank_zero_only(orc):
    assert _run({"WORLD_SIZE": "2", "RANK": "1", "LOCAL_RANK": "1"}) == []
