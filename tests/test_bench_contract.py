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


def test_profile_records_the_bench_reads():
    """The roofline inputs bench.py reads from profiles/: the DRAM bytes of
    the bench launch itself (a one-pass capture of 1024 columns x 120 steps)
    and the FP64 form's FP64 warp-instructions per column-step."""
    with open(os.path.join(REPO, 'profiles', 'crm_columns_fp32_traffic.json')) as f:
        tr = json.load(f)
    assert tr['passes'] == 1 and tr['column_steps_in_capture'] == 1024 * 120
    assert tr['bytes_per_launch'] == tr['dram_bytes_read'] + tr['dram_bytes_write']
    # more than the algorithmic bytes (27 words per cell, 4 B), far below a
    # re-read of the whole slab every phase
    assert tr['algorithmic_bytes_per_launch'] == 1024 * 120 * 27 * 64 * 58 * 4
    assert 1.0 < tr['bytes_per_launch'] / tr['algorithmic_bytes_per_launch'] < 20.0
    with open(os.path.join(REPO, 'profiles', 'crm_columns_fp64_pipe.json')) as f:
        fp = json.load(f)
    assert fp['passes'] == 1
    assert abs(fp['fp64_warp_inst_per_column_step'] * fp['column_steps_in_capture'] - fp['fp64_warp_instructions']) < 1.0
