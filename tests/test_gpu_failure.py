"""Failure detection on the GPU, with no GPU fault: a non-finite column is
reported per column and leaves its batch-mates' bits alone, and a grid
barrier whose arrival never comes gives up and reports CRM_ERR_TIMEOUT with
the context still usable."""
import numpy as np
import pytest

import oracle
from crm_gb300 import crm_types as T
from crm_gb300 import synthetic as S
from crm_gb300.lib import CrmContext

pytestmark = pytest.mark.gpu


def _gpu(cfg, cin, st, rad, desc, ctx=None):
    cfg.max_ncrms = max(cfg.max_ncrms, desc.ld)
    ctx = ctx or CrmContext(cfg)
    out = T.CrmOutput(desc.ld, cfg.crm_nx, cfg.crm_ny, cfg.crm_nz, cfg.plev)
    st, rad = st.copy(), rad.copy()
    stat = ctx.run(desc, cin, st, rad, out)
    return ctx.last_rc, stat, (st, rad, out)


def _same_columns(a, b, cols):
    for x, y in zip(a, b):
        for n, v in x.arrays().items():
            assert np.array_equal(v[cols], getattr(y, n)[cols]), n


@pytest.mark.parametrize('precision', [T.CRM_FP64, T.CRM_FP32_MIXED])
def test_nonfinite_column_reported_others_unchanged(gpu_lib, precision):
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=4, precision=precision)
    desc.dt_gl = 200.0
    bad = st.copy()
    bad.temperature[2, 9, 0, 3] = np.nan
    rc, stat, res_b = _gpu(cfg, cin, bad, rad, desc)
    assert rc == T.CRM_ERR_NONFINITE
    assert list(stat) == [0, 0, T.CRM_ERR_NONFINITE, 0]
    rc, stat, res_g = _gpu(cfg, cin, st, rad, desc)
    assert rc == 0
    _same_columns(res_b, res_g, [0, 1, 3])
    if precision == T.CRM_FP64:    # the oracle stops the same column with the same bits
        st_o, rad_o = bad.copy(), rad.copy()
        rc_o, stat_o, out_o = oracle.run(cfg, desc, cin, st_o, rad_o)
        assert list(stat_o) == [0, 0, T.CRM_ERR_NONFINITE, 0]
        _same_columns(res_b, (st_o, rad_o, out_o), [0, 1, 3])


def test_nonfinite_input_profile_stops_a_reference_batch(gpu_lib):
    """A NaN in one column's GCM input (tl) in reference-batch mode: that
    column reports CRM_ERR_NONFINITE, the rest of the batch CRM_ERR_CFL, as
    the oracle's batch mode does; nobody waits at the grid barrier."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=4, batch_mode=T.CRM_REFERENCE_BATCH)
    desc.dt_gl = 200.0
    cin = cin.copy()
    cin.tl[1, cfg.plev - 3] = np.nan
    rc, stat, _ = _gpu(cfg, cin, st, rad, desc)
    st_o = st.copy()
    rc_o, stat_o, _ = oracle.run(cfg, desc, cin, st_o, rad.copy())
    want = [T.CRM_ERR_CFL, T.CRM_ERR_NONFINITE, T.CRM_ERR_CFL, T.CRM_ERR_CFL]
    assert list(stat) == want and list(stat_o) == want


def test_grid_barrier_wait_runs_out(gpu_lib):
    """Reference-batch mode with one column withholding its arrival at the
    first grid barrier and a short wait limit: every column reports
    CRM_ERR_TIMEOUT, the call returns, and the next call on the same handle
    (normal arrivals) matches the oracle bit for bit."""
    import time
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=6, batch_mode=T.CRM_REFERENCE_BATCH)
    desc.dt_gl = 200.0
    cfg.max_ncrms = desc.ld
    ctx = CrmContext(cfg)
    assert gpu_lib.crm_debug_barrier_test(ctx._h, 1 << 12, 2) == 0
    t0 = time.perf_counter()
    rc, stat, _ = _gpu(cfg, cin, st, rad, desc, ctx)
    assert time.perf_counter() - t0 < 30.0
    assert rc == T.CRM_ERR_TIMEOUT
    assert list(stat) == [T.CRM_ERR_TIMEOUT] * 6
    assert gpu_lib.crm_debug_barrier_test(ctx._h, 1 << 24, -1) == 0
    rc, stat, (st_g, rad_g, out_g) = _gpu(cfg, cin, st, rad, desc, ctx)
    assert rc == 0 and not stat.any()
    st_o, rad_o = st.copy(), rad.copy()
    rc_o, _, out_o = oracle.run(cfg, desc, cin, st_o, rad_o)
    assert rc_o == 0
    _same_columns((st_g, rad_g, out_g), (st_o, rad_o, out_o), slice(None))
