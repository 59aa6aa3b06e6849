"""bench.py's reference arm (the oracle restatement of compute_Ku,
tests/test_bri17.cpp:56-107, timed on the host cores) prints one JSON line
with the keys of the bench contract, on CPU; under torchrun only rank 0
prints it and the other ranks exit 0 without work."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KEYS = ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
        "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
        "cpu_baseline", "e2e")


def _run(env_extra, *args):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, "bench.py", "--impl", "reference", *args],
                          cwd=REPO, env=env, capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_one_contract_line():
    p = _run({}, "--steps", "1", "--warmup", "3")
    assert p.returncode == 0, p.stderr
    lines = [ln for ln in p.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    for k in KEYS:
        assert k in d, k
    assert d["impl"] == "reference" and d["unit"] == "GDoF/s"
    assert d["steps"] == 1 and d["warmup"] == 3 and d["value"] > 0
    assert d["higher_is_better"] is True and d["dtype"] == "f64"
    assert d["config"]["grid"] == [128, 128, 128]
    assert d["config"]["dof_per_step"] == 3 * 128 ** 3
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "GDoF/s",
                        "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # value = DoF per step / time per step.
    assert abs(d["value"] - 3 * 128 ** 3 / (d["ms_per_step"] * 1e-3) / 1e9) <= 1e-9 * d["value"]


def test_reference_arm_other_ranks_exit_without_work():
    p = _run({"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"},
             "--gpus", "2", "--steps", "1", "--warmup", "3")
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""


def test_reference_arm_follows_shape_and_names_unavailable_workloads():
    for shape in ("32x32x32", "64x64"):
        p = _run({}, "--shape", shape, "--steps", "1", "--warmup", "3")
        assert p.returncode == 0, p.stderr
        d = json.loads(p.stdout.strip().splitlines()[-1])
        dims = [int(n) for n in shape.split("x")]
        assert d["config"]["grid"] == dims
        assert d["config"]["dof_per_step"] == len(dims) * int(__import__("math").prod(dims))
        assert shape in d["cpu_baseline"]["sample"]
    for workload in ("cg", "aniso", "serve"):
        p = _run({}, "--workload", workload, "--steps", "1", "--warmup", "3")
        assert p.returncode == 0, p.stderr
        d = json.loads(p.stdout.strip())
        assert d["impl"] == "reference" and "unavailable" in d and workload in d["unavailable"]
