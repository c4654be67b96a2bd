"""CRM_FP64_FMA: the FP64 form compiled with multiply-add contraction.  Its
roundings differ from the oracle's (which keeps every multiply and add
separate), so it is held to the plain form's tolerance of 1e-10 relative L2
on every state, rad and output field after a GCM step."""
import numpy as np
import pytest

import oracle
from crm_gb300 import synthetic as S
from crm_gb300 import crm_types as T
from crm_gb300.lib import CrmContext

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _worst(cfg, cin, st, rad, desc):
    st_o, rad_o = st.copy(), rad.copy()
    rc, _, out_o = oracle.run(cfg, desc, cin, st_o, rad_o)
    assert rc == 0
    c = T.CrmConfig(**{**cfg.__dict__, 'precision': T.CRM_FP64_FMA, 'max_ncrms': desc.ld})
    ctx = CrmContext(c)
    out = T.CrmOutput(desc.ld, c.crm_nx, c.crm_ny, c.crm_nz, c.plev)
    st_g, rad_g = st.copy(), rad.copy()
    ctx.run(desc, cin, st_g, rad_g, out, raise_on_error=True)
    errs = [(rel_l2(getattr(st_g, n), x), 'state.' + n) for n, x in st_o.arrays().items()]
    errs += [(rel_l2(getattr(rad_g, n), getattr(rad_o, n)), 'rad.' + n)
             for n in ('temperature', 'qv', 'qc', 'qi', 'cld')]
    errs += [(rel_l2(getattr(out, n), x), 'out.' + n) for n, x in out_o.arrays().items()]
    return max(errs)


@pytest.mark.parametrize('moist', [False, True])
def test_fp64_fma_64x58_within_1e10(gpu_lib, moist):
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=4, moist=moist)
    worst = _worst(cfg, cin, st, rad, desc)
    print('FP64 with contraction, 64x58 (moist=%s): worst field' % moist, worst)
    assert worst[0] <= TOL, worst


def test_fp64_fma_32x28_moist_within_1e10(gpu_lib):
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=4, moist=True)
    worst = _worst(cfg, cin, st, rad, desc)
    assert worst[0] <= TOL, worst


def test_fp64_fma_3d_within_1e10(gpu_lib):
    cfg, cin, st, rad, desc = S.workload_3d(ncrms=2, nx=16, ny=16, moist=True)
    desc.dt_gl = 300.0
    worst = _worst(cfg, cin, st, rad, desc)
    print('FP64 with contraction, 3D 16x16x58: worst field', worst)
    assert worst[0] <= TOL, worst
