"""bench.py's reference arm (the reference algorithm on the host cores) runs
without a GPU and prints one JSON line with the contract's keys."""
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    t0 = time.perf_counter()
    out = subprocess.run([sys.executable, 'bench.py', '--impl', 'reference', '--steps', '4', '--warmup', '3'],
                         cwd=ROOT, capture_output=True, text=True, timeout=600)
    wall = time.perf_counter() - t0
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip().startswith('{')]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ('metric', 'value', 'unit', 'n_gpus', 'steps', 'warmup', 'ms_per_step', 'higher_is_better',
                'scaling', 'vs_baseline', 'dtype', 'data', 'config', 'impl', 'cpu_baseline', 'e2e'):
        assert key in d, key
    assert d['impl'] == 'reference' and d['value'] > 0 and d['higher_is_better'] is True
    assert d['unit'] == 'instance-steps/s' and d['config']['workload']
    cb = d['cpu_baseline']
    assert cb['value'] == d['value'] and cb['kind'] in ('port', 'reference') and cb['cores'] >= 1 and cb['sample']
    assert d['e2e'] == {'value': d['value'], 'unit': d['unit'], 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}
    # the line describes its own sample: the K timed steps fit inside the run
    assert d['steps'] == 4 and d['warmup'] == 3
    assert d['steps'] * d['ms_per_step'] / 1e3 < wall
    # value = instance-steps per second of the timed steps
    inner = int(d['config']['arm_step'].split()[0])
    per_step = inner * cb['cores']
    assert abs(d['value'] - per_step / (d['ms_per_step'] / 1e3)) < 1e-6 * d['value']
