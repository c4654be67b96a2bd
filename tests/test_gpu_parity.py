"""FP64 device form against the CPU restatement, through the C ABI.

Both evaluate the same IEEE operations in the same order (no FMA contraction,
deterministic exp/log/pow, horizontal sums in the reference's loop order), so
every state, rad and output field must agree bit for bit.
"""
import numpy as np
import pytest

import oracle
from crm_gb300 import synthetic as S
from crm_gb300 import types as T
from crm_gb300.lib import CrmContext

pytestmark = pytest.mark.gpu


def _run_both(cfg, cin, st, rad, desc):
    st_o, rad_o = st.copy(), rad.copy()
    rc, stat_o, out_o = oracle.run(cfg, desc, cin, st_o, rad_o)
    assert rc == 0, stat_o
    cfg.max_ncrms = desc.ld
    ctx = CrmContext(cfg)
    st_g, rad_g = st.copy(), rad.copy()
    out_g = T.CrmOutput(desc.ld, cfg.crm_nx, cfg.crm_ny, cfg.crm_nz, cfg.plev)
    stat_g = ctx.run(desc, cin, st_g, rad_g, out_g)
    assert ctx.last_rc == 0, stat_g
    return (st_o, rad_o, out_o), (st_g, rad_g, out_g)


def _compare_exact(a, b):
    bad = []
    for name in ('st', 'rad', 'out'):
        pass
    (st_o, rad_o, out_o), (st_g, rad_g, out_g) = a, b
    for n, x in st_o.arrays().items():
        y = getattr(st_g, n)
        if not np.array_equal(x, y):
            bad.append(('state.' + n, float(np.max(np.abs(x - y)))))
    for n in ('temperature', 'qv', 'qc', 'qi', 'cld'):
        x, y = getattr(rad_o, n), getattr(rad_g, n)
        if not np.array_equal(x, y):
            bad.append(('rad.' + n, float(np.max(np.abs(x - y)))))
    for n, x in out_o.arrays().items():
        y = getattr(out_g, n)
        if not np.array_equal(x, y):
            bad.append(('out.' + n, float(np.max(np.abs(x - y)))))
    return bad


def test_fp64_bitexact_workload0_short(gpu_lib):
    cfg, cin, st, rad, desc = S.workload0(ncrms=4)
    desc.dt_gl = 200.0          # 10 CRM steps
    a, b = _run_both(cfg, cin, st, rad, desc)
    assert _compare_exact(a, b) == []


def test_fp64_bitexact_workload0_full(gpu_lib):
    cfg, cin, st, rad, desc = S.workload0(ncrms=16)
    a, b = _run_both(cfg, cin, st, rad, desc)
    assert _compare_exact(a, b) == []
