"""bench.py's command-line contract, on the CPU: the reference arm (ZodiPy's numpy path on
the host cores) prints one JSON line with the keys the GPU arm prints, on the same workload;
under a multi-rank launch only rank 0 runs it."""

import json
import os
import subprocess
import sys

from conftest import REPO


def _run_bench(*args, env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run(
        [sys.executable, os.path.join(REPO, "bench.py"), *args],
        cwd=REPO,
        env=env,
        capture_output=True,
        text=True,
        timeout=600,
    )


def test_reference_arm_prints_one_contract_line():
    r = _run_bench("--impl", "reference", "--steps", "1", "--warmup", "0", "--nside", "64")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["unit"] == "LOS/s" and d["value"] > 0
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    sys.path.insert(0, REPO)
    import bench

    assert d["config"] == bench.bench_config(64)  # the GPU arm reports the same config
    assert d["config"]["los_per_step"] == 12 * 64 * 64
    assert d["metric"] == bench.METRIC


def test_reference_arm_does_not_touch_the_package():
    """The reference arm runs the oracle on reference-held data: after it, no module of the
    package is imported and the package's shared library is not mapped."""
    code = (
        "import runpy, sys\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', '--nside', '16']\n"
        "runpy.run_path('bench.py', run_name='__main__')\n"
        "mods = sorted(m for m in sys.modules if m.startswith('zodipy_gb300'))\n"
        "maps = open('/proc/self/maps').read()\n"
        "assert not mods, mods\n"
        "assert 'libzodigb' not in maps\n"
        "print('clean')\n"
    )
    r = subprocess.run([sys.executable, "-c", code], cwd=REPO, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().splitlines()[-1] == "clean"


def test_reference_arm_runs_on_rank_zero_only():
    r = _run_bench("--impl", "reference", "--steps", "1", "--warmup", "0", "--nside", "64",
                   env_extra={"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
