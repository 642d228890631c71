"""bench.py --impl reference (the CPU oracle on the host cores) prints the
JSON line the benchmark contract asks for, and non-zero ranks exit without
work.  Runs a tiny sample: the half cell at refinement 4, two oracle
processes, one timed step each."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(extra_env=None, gpus=1, rc=0):
    env = dict(os.environ, **(extra_env or {}))
    if "WORLD_SIZE" not in (extra_env or {}):
        env.pop("WORLD_SIZE", None)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", str(gpus), "--steps", "2", "--warmup", "1", "--cpu-sample-steps", "1",
                        "--ref-procs", "2", "--refine", "4"], capture_output=True, text=True, env=env,
                       timeout=600)
    assert r.returncode == rc, r.stderr
    return [l for l in r.stdout.splitlines() if l.startswith("{")]


def test_reference_arm_json_line():
    lines = _run()
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert "2x16x16" in d["config"]["workload"]
    assert d["metric"] == "I-V points/sec to steady state" and d["unit"] == "I-V points/s"
    cb = d["cpu_baseline"]
    assert cb["cores"] == 2 and cb["kind"] == "port" and cb["value"] == d["value"]
    assert set(cb) >= {"value", "unit", "cores", "kind", "sample"}
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    # ms_per_step is the measured time of one bench step (one IMEX step of each
    # process here); points/sec is derived from it and the steps to steady state
    c = d["config"]
    assert abs(d["ms_per_step"] - c["ms_per_imex_step"]) < 1e-9 * d["ms_per_step"]
    want = 2 / (c["steps_to_steady_state"] * c["ms_per_imex_step"] * 1e-3)
    assert abs(d["value"] - want) < 1e-9 * want
    assert c["steps_to_steady_state_source"]


def test_reference_arm_other_ranks_do_nothing():
    assert _run({"RANK": "1", "WORLD_SIZE": "2"}, gpus=2) == []


def test_gpu_count_must_match_the_launcher():
    """--gpus N without N launched ranks is refused instead of silently
    running one rank."""
    assert _run(gpus=2, rc=2) == []
    assert _run({"RANK": "0", "WORLD_SIZE": "2"}, gpus=1, rc=2) == []
