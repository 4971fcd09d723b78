"""bench.py's contract where no GPU is needed: the reference arm (WFA2-lib, or the oracle where
WFA2-lib's sources are absent, on the host cores) prints one JSON line with the keys the line
format asks for; a rank other than 0 prints nothing and exits 0; and the GPU arm fails loudly
without a device instead of falling back to the CPU."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _bench(*args, env=None, timeout=600):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], cwd=ROOT, env=e, capture_output=True,
                          text=True, timeout=timeout)


def test_reference_arm_prints_one_contract_line():
    r = _bench("--impl", "reference", "--steps", "1", "--warmup", "3", "--pairs", "600")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "pairs/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] >= 3
    assert d["config"]["num_pairs"] == 600 and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert isinstance(cb["cpu"], str) and cb["cpu"]
    assert d["e2e"] == {"value": d["value"], "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    r = _bench("--impl", "reference", "--steps", "1", "--warmup", "3", "--pairs", "600",
               env={"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_gpu_arm_fails_without_a_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    r = _bench("--steps", "1", "--warmup", "3", "--pairs", "200", "--no-cpu-baseline", timeout=300)
    assert r.returncode != 0
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{") and '"value"' in ln]
    assert "no usable CUDA device" in r.stderr


def test_host_cpu_names_the_machine():
    sys.path.insert(0, str(ROOT))
    import bench
    import platform
    assert bench.host_cpu().endswith(platform.machine() + ")") or bench.host_cpu() == platform.machine()
