"""The benchmark's reference arm on the host: `bench.py --impl reference`
prints one JSON line with the contract's keys (the metric and config of the
GPU arm, a cpu_baseline describing the run, an e2e block with no transfers).
Runs the CPU restatement of the reference on one short step (no GPU)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_contract():
    env = dict(os.environ)
    env.pop('RANK', None)
    env.pop('WORLD_SIZE', None)
    out = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--steps', '1',
                          '--warmup', '0'], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip().startswith('{')]
    assert len(lines) == 1, out.stdout[-2000:]
    d = json.loads(lines[0])
    assert d['impl'] == 'reference'
    for key in ('metric', 'value', 'unit', 'steps', 'warmup', 'ms_per_step', 'higher_is_better', 'dtype',
                'config', 'cpu_baseline', 'e2e'):
        assert key in d, key
    assert d['value'] > 0 and d['unit'] == 'evals/s' and d['higher_is_better'] is True
    assert d['steps'] == 1 and d['warmup'] == 0
    assert 'workload' in d['config']
    cb = d['cpu_baseline']
    assert cb['value'] == d['value'] and cb['unit'] == d['unit']
    assert cb['kind'] in ('reference', 'port') and cb['cores'] >= 1 and cb['sample']
    e2e = d['e2e']
    assert e2e['value'] == d['value'] and e2e['h2d_bytes_per_step'] == 0 and e2e['d2h_bytes_per_step'] == 0
