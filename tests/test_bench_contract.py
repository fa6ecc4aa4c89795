"""The JSON line of `bench.py --impl reference` (the CPU reference arm) at small sizes, on the host:
one line with the contract's keys, the oracle timed as the reference (`kind` "port"), no device
traffic in `e2e`; ranks other than 0 print nothing and exit 0; the GPU arm exits non-zero where
there is no GPU instead of falling back to the CPU."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = {"metric", "value", "unit", "impl", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"}


def run_bench(argv, env=None, timeout=240):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + argv, cwd=ROOT, env=e,
                          capture_output=True, text=True, timeout=timeout)


@pytest.fixture(scope="module", autouse=True)
def built_oracle(oracle):
    return oracle


@pytest.mark.parametrize("workload,n", [("grid", 128), ("sr", 48), ("gr", 32)])
def test_reference_arm_prints_one_contract_line(workload, n):
    r = run_bench(["--workload", workload, "--impl", "reference", "--n", str(n), "--steps", "1", "--warmup", "3"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert KEYS <= set(line)
    assert line["impl"] == "reference"
    assert line["metric"] == line["unit"] == "cell-updates/s"
    assert line["higher_is_better"] is True and line["vs_baseline"] is None
    assert line["steps"] == 1 and line["warmup"] == 3 and line["n_gpus"] == 1
    assert line["config"]["n"] == n
    assert line["value"] > 0
    assert line["ms_per_step"] == pytest.approx(n * n / line["value"] * 1e3, rel=1e-9)
    base = line["cpu_baseline"]
    assert base["kind"] == "port" and base["cores"] >= 1 and base["sample"]
    assert base["value"] == line["value"] and base["unit"] == line["unit"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    if workload == "grid":  # both arms print the same config dict for the headline workload
        sys.path.insert(0, ROOT)
        import bench
        assert line["config"] == bench.grid_config(n, 1)
        assert "1 timed" in base["sample"] and "3 untimed" in base["sample"]


@pytest.mark.parametrize("workload", ["sod", "batch"])
def test_single_config_reference_arms(workload):
    r = run_bench(["--workload", workload, "--impl", "reference", "--steps", "1", "--warmup", "3"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert KEYS <= set(line) and line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0


def test_conservation_totals():
    sys.path.insert(0, ROOT)
    import bench
    rng = np.random.default_rng(3)
    p = np.stack([rng.uniform(0.5, 1.5, (8, 9)), rng.uniform(-0.3, 0.3, (8, 9)), rng.uniform(-0.3, 0.3, (8, 9)),
                  np.zeros((8, 9)), rng.uniform(0.1, 1.0, (8, 9))], axis=-1)
    m, e = bench.newton_totals(p, 1.4)
    assert m == pytest.approx(p[..., 0].sum(), rel=1e-15)
    v2 = (p[..., 1:4] ** 2).sum(-1)
    assert e == pytest.approx((0.5 * p[..., 0] * v2 + p[..., 4] / 0.4).sum(), rel=1e-14)
    d, tau = bench.sr_totals(p, 5.0 / 3.0)
    W = 1.0 / np.sqrt(1.0 - v2)
    h = 1.0 + p[..., 4] / p[..., 0] * 2.5
    assert d == pytest.approx((p[..., 0] * W).sum(), rel=1e-14)
    assert tau == pytest.approx((p[..., 0] * h * W * W - p[..., 4] - p[..., 0] * W).sum(), rel=1e-14)
    assert bench.drift((2.0, 4.0), (2.0 + 2e-7, 4.0 - 4e-6)) == pytest.approx({"mass": 1e-7, "energy": 1e-6})
    assert bench.rel_l1(np.array([1.0, 2.0]), np.array([1.0, 1.0])) == pytest.approx(0.5)


def test_amr_reference_arm_prints_one_contract_line():
    r = run_bench(["--workload", "amr", "--impl", "reference", "--n", "64", "--steps", "1"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert KEYS <= set(line) and line["impl"] == "reference" and line["value"] > 0
    assert line["config"]["n"] == 64 and line["ms_per_step"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and "coarse" in line["cpu_baseline"]["sample"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    r = run_bench(["--impl", "reference", "--n", "64", "--steps", "1", "--gpus", "2"],
                  env={"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def test_gpu_arm_fails_without_a_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = run_bench(["--n", "64", "--steps", "1", "--no-cpu"])
    assert r.returncode != 0
    assert r.stdout.strip() == ""
