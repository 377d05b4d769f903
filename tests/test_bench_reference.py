"""The reference arm of bench.py (`--impl reference`): the oracle's CPU
restatement on tiny workloads prints one JSON line with the fields the
benchmark contract needs (impl, metric, value, unit, cpu_baseline with kind
and cores, e2e with zero copy bytes)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("config,refs", [("c3", 600), ("c5", 1200)])
def test_reference_arm_json(config, refs):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config", config,
                        "--refs", str(refs), "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "reads/s" and d["value"] > 0
    assert d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert "reads/s" in d["metric"]


def test_reference_arm_maps_no_gpu_library():
    """The reference arm builds its workload with libhdc_synth.so and the oracle
    only: libhdc_gb300.so (the product) is never mapped into its process."""
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--config', 'c3', '--refs', '300', "
            "'--steps', '1', '--warmup', '3']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('MAPS', 'libhdc_gb300' in maps, 'libhdc_synth' in maps, 'liboracle' in maps)")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "MAPS False True True" in r.stdout


def test_multi_gpu_launch_is_declined():
    """The library is single-GPU: under a multi-process launch rank 0 prints an
    'unavailable' line, no work is done and every rank exits 0."""
    for rank in ("0", "1"):
        env = dict(os.environ, WORLD_SIZE="2", RANK=rank, LOCAL_RANK=rank)
        r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2"], capture_output=True,
                           text=True, timeout=120, cwd=ROOT, env=env)
        assert r.returncode == 0, r.stderr[-2000:]
        lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
        if rank == "0":
            assert len(lines) == 1 and "unavailable" in json.loads(lines[0])
        else:
            assert not lines
