"""bench.py's reference arm on the host (no GPU needed): one JSON line with
the fields of the benchmark contract, the same metric and workload config as
the GPU arm, and zero host<->device bytes."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    env = dict(os.environ, CRM_BENCH_CPU_COLS='2')
    r = subprocess.run([sys.executable, os.path.join(REPO, 'bench.py'), '--impl', 'reference',
                        '--steps', '1', '--warmup', '0'],
                       capture_output=True, text=True, env=env, cwd=REPO, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ('metric', 'value', 'unit', 'n_gpus', 'steps', 'warmup', 'ms_per_step',
                'higher_is_better', 'scaling', 'vs_baseline', 'dtype', 'data', 'config',
                'cpu_baseline', 'e2e'):
        assert key in line, key
    assert line['impl'] == 'reference'
    assert line['value'] > 0 and line['higher_is_better'] is True
    assert line['config']['ncrms'] == 1024 and line['config']['nstop'] == 120
    cb = line['cpu_baseline']
    assert set(cb) >= {'value', 'unit', 'cores', 'kind', 'sample'} and cb['kind'] == 'port'
    e2e = line['e2e']
    assert e2e['h2d_bytes_per_step'] == 0 and e2e['d2h_bytes_per_step'] == 0
    assert e2e['value'] == line['value'] and e2e['unit'] == line['unit']
