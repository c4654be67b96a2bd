"""Regenerate the oracle fixtures in this directory.

    python tests/golden/make_golden.py

The reference ships no stored CRM inputs or outputs, so these fixtures pin
the CPU restatement (oracle/) against itself: seeded synthetic inputs
(acme-ecp_gb300/crm_gb300/synthetic.py), one crm() call, and the resulting
state, radiation means and GCM tendencies.  test_golden.py recomputes them
and must reproduce them bit for bit on the platform that wrote them (host
libm functions enter the FFT tables and gamma constants, so another
platform is held to 1e-9 relative instead).
"""
import hashlib
import os
import platform
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, 'acme-ecp_gb300'))
sys.path.insert(0, os.path.join(REPO, 'oracle'))

OUT_FIELDS = ('precc', 'precl', 'cltot', 'sltend', 'qltend', 'qcltend', 'qiltend', 'prectend',
              'cld', 'mcup', 'flux_qt', 'tkez', 'qc_mean', 'qi_mean', 'qr_mean', 'jt_crm', 'z0m')

CASES = {
    # name: (workload, kwargs, dt_gl)
    'w32x28_moist_2col': ('workload_32x28', {'ncrms': 2, 'moist': True}, 400.0),
    'w64x58_moist_1col': ('workload_64x58', {'ncrms': 1, 'moist': True}, 100.0),
}


def inputs_hash(cin, st, rad):
    h = hashlib.sha256()
    for b in (cin, st, rad):
        for n, a in b.arrays().items():
            h.update(n.encode())
            h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def run_case(name):
    import oracle
    from crm_gb300 import synthetic as S
    wl, kw, dt_gl = CASES[name]
    cfg, cin, st, rad, desc = getattr(S, wl)(**kw)
    desc.dt_gl = dt_gl
    h = inputs_hash(cin, st, rad)
    rc, stat, out = oracle.run(cfg, desc, cin, st, rad, nthreads=1)
    assert rc == 0, stat
    res = {'inputs_sha256': np.array(h)}
    for n, a in st.arrays().items():
        res['state.' + n] = a
    for n in ('temperature', 'qv', 'qc', 'qi', 'cld'):
        res['rad.' + n] = getattr(rad, n)
    for n in OUT_FIELDS:
        res['out.' + n] = getattr(out, n)
    return res


def main():
    for name in CASES:
        res = run_case(name)
        res['platform'] = np.array('%s-%s' % (platform.system(), platform.machine()))
        np.savez_compressed(os.path.join(HERE, name + '.npz'), **res)
        print('wrote', name)


if __name__ == '__main__':
    main()
