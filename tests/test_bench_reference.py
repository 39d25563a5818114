"""CPU test of the bench contract's reference arm (the oracle on the host
cores; no GPU): one JSON line with the metric, the CPU baseline block and a
zero-copy e2e block; timing rules enforced on the command line."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _bench(*args, env_extra=None, timeout=600):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=timeout)


def test_reference_arm_prints_one_contract_line():
    r = _bench("--impl", "reference", "--steps", "1", "--warmup", "3", env_extra={"SDT_CPU_FLOP_CAP": "4e10"})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "(T) TFLOP/s" and d["unit"] == "TFLOP/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 3
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["config"] == {"workload": d["config"]["workload"], "form": "fp64"}
    assert d["e2e"] == {"value": d["value"], "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_too_few_warmup_steps_are_refused():
    r = _bench("--impl", "reference", "--steps", "1", "--warmup", "1", timeout=120)
    assert r.returncode == 2 and "warmup" in r.stderr


def test_reference_arm_does_not_load_the_product_library():
    """The reference arm builds its inputs, tuple list and FLOP counts on the
    checker side: the product library is never loaded."""
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3'];"
            "import os; os.environ['SDT_CPU_FLOP_CAP'] = '4e10';"
            "runpy.run_path('bench.py', run_name='__main__');"
            "maps = open('/proc/self/maps').read();"
            "assert 'libsdt_gb300' not in maps and 'libsdt_oracle' in maps, 'library check'")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]


def test_reference_sample_is_uniform_over_the_slice():
    """The sampled tuples are drawn from the whole slice (seeded), not its
    smallest tuples."""
    import numpy as np
    sys.path.insert(0, str(ROOT))
    import bench
    sl = np.arange(5, 2860, 256)
    picks = np.concatenate([bench.ref_sample(sl, s) for s in range(200)])
    assert set(picks.tolist()) <= set(sl.tolist()) and len(set(picks.tolist())) == len(sl)
    assert np.array_equal(bench.ref_sample(sl, 7), bench.ref_sample(sl, 7))


def test_reference_arm_other_ranks_exit_quietly():
    """Under torchrun with N > 1 only rank 0 runs the reference arm and
    prints its line; the other ranks exit 0 without work or output."""
    r = _bench("--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3",
               env_extra={"WORLD_SIZE": "2", "RANK": "1", "LOCAL_RANK": "1"}, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
