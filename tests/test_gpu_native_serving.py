"""The C-ABI serving entry points (crm_server_create, crm_chunk_open,
crm_submit, crm_poll) on the GPU, through ctypes as a C or Fortran host
would call them: a chunk's results are the same alone and batched with
other chunks' concurrent steps, equal a direct crm_run, and a chunk's two
steps submitted back to back equal the same steps run one after the
other."""
import numpy as np
import pytest

from crm_gb300 import crm_types as T
from crm_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

DT_GL = 300.0
STEP = ('sltend', 'qltend', 'qcltend', 'qiltend', 'precc', 'precl', 'cltot', 'prectend', 'tk', 'cld')


def _cfg():
    return T.CrmConfig(crm_nx=32, crm_ny=1, crm_nz=28, plev=72, crm_dx=1000.0, crm_dt=10.0,
                       precision=T.CRM_FP32_MIXED)


def _chunk(cfg, ncol, gcol0, seed):
    from crm_gb300.serve_bench import make_chunk
    return make_chunk(cfg, ncol, gcol0, seed)


def _vals(t):
    return {n: getattr(t.out, n).copy() for n in STEP}


def test_native_chunk_alone_equals_chunk_in_mix(gpu_lib):
    from crm_gb300.native_server import NativeCrmServer
    cfg = _cfg()
    a = _chunk(cfg, 5, 101, seed=7)
    others = [_chunk(cfg, 3 + 9 * i, 1000 * (i + 1), seed=i) for i in range(4)]
    srv = NativeCrmServer(cfg, capacity=128)
    ca = srv.open_chunk(a[1], a[2], a[3])
    alone = []
    for _ in range(2):
        t = srv.submit(ca, a[0], 5, DT_GL, fields=STEP)
        assert t.poll() == 0
        alone.append(_vals(t))
    srv.close_chunk(ca)
    # the same chunk again, now submitted together with four other chunks
    ca = srv.open_chunk(a[1], a[2], a[3])
    cs = [srv.open_chunk(o[1], o[2], o[3]) for o in others]
    mixed = []
    for _ in range(2):
        ts = [srv.submit(c, o[0], len(o[3]), DT_GL, fields=STEP) for c, o in zip(cs, others)]
        ta = srv.submit(ca, a[0], 5, DT_GL, fields=STEP)
        assert ta.poll() == 0 and all(t.poll() == 0 for t in ts)
        mixed.append(_vals(ta))
    launches = srv.launches
    srv.close()
    assert launches <= 2 + 2 * 5 - 1      # some steps of different chunks shared a launch
    for s in range(2):
        for n in STEP:
            assert np.array_equal(alone[s][n], mixed[s][n]), (s, n)


def test_native_step_equals_crm_run(gpu_lib):
    """First step through the service == crm_run of the same columns, for
    every crm_output field, the rad means and the returned state."""
    from crm_gb300.lib import CrmContext
    from crm_gb300.native_server import NativeCrmServer
    cfg = _cfg()
    cin, st, rad, gcol = _chunk(cfg, 6, 11, seed=3)
    srv = NativeCrmServer(cfg, capacity=32, handles=2)
    c = srv.open_chunk(st, rad, gcol)
    t = srv.submit(c, cin, 6, DT_GL, rad_means=True)
    assert t.poll() == 0 and not t.status.any()
    st_dev, qrad_dev = srv.read_state(c, 6)
    srv.close()
    c2 = T.CrmConfig(**{**cfg.__dict__, 'max_ncrms': 6})
    ctx = CrmContext(c2)
    out = T.CrmOutput(6, cfg.crm_nx, 1, cfg.crm_nz, cfg.plev)
    desc = T.call_desc(6, 6, DT_GL, 1, gcol)
    st2, rad2 = st.copy(), rad.copy()
    status = ctx.run(desc, cin, st2, rad2, out)
    assert not status.any()
    for n, v in out.arrays().items():
        assert np.array_equal(v, getattr(t.out, n)), n
    for n in ('temperature', 'qv', 'qc', 'qi', 'cld'):
        assert np.array_equal(getattr(rad2, n), getattr(t.rad, n)), n
    for n, v in st2.arrays().items():
        assert np.array_equal(v, getattr(st_dev, n)), n
    assert np.array_equal(qrad_dev, rad.qrad)


def test_native_back_to_back_steps_of_one_chunk(gpu_lib):
    from crm_gb300.native_server import NativeCrmServer
    cfg = _cfg()
    cin, st, rad, gcol = _chunk(cfg, 4, 51, seed=5)
    srv = NativeCrmServer(cfg, capacity=16)
    c = srv.open_chunk(st, rad, gcol)
    seq = []
    for _ in range(2):
        t = srv.submit(c, cin, 4, DT_GL, fields=STEP)
        assert t.poll() == 0
        seq.append(_vals(t))
    srv.close_chunk(c)
    c = srv.open_chunk(st, rad, gcol)
    t1 = srv.submit(c, cin, 4, DT_GL, fields=STEP)
    t2 = srv.submit(c, cin, 4, DT_GL, fields=STEP)
    assert t2.poll() == 0 and t1.poll() == 0
    srv.close()
    for s, t in enumerate((t1, t2)):
        for n in STEP:
            assert np.array_equal(seq[s][n], getattr(t.out, n)), (s, n)
    assert not np.array_equal(seq[0]['sltend'], seq[1]['sltend'])


def test_native_admission_limits(gpu_lib):
    """A budget too small for the pool refuses the server with
    CRM_ERR_BUDGET; a chunk larger than the free slots is refused with
    CRM_ERR_BUDGET and admitted once another chunk closes."""
    from crm_gb300.lib import CrmError
    from crm_gb300.native_server import NativeCrmServer
    cfg = _cfg()
    with pytest.raises(CrmError) as e:
        NativeCrmServer(cfg, capacity=64, hbm_budget=1 << 20)
    assert e.value.status == T.CRM_ERR_BUDGET
    srv = NativeCrmServer(cfg, capacity=8)
    assert 0 < srv.device_bytes <= 120 * 2 ** 30
    a = _chunk(cfg, 6, 1, seed=1)
    b = _chunk(cfg, 4, 7, seed=2)
    ca = srv.open_chunk(a[1], a[2], a[3])
    with pytest.raises(CrmError) as e:
        srv.open_chunk(b[1], b[2], b[3])
    assert e.value.status == T.CRM_ERR_BUDGET
    srv.close_chunk(ca)
    cb = srv.open_chunk(b[1], b[2], b[3])
    t = srv.submit(cb, b[0], 4, DT_GL, fields=STEP)
    assert t.poll() == 0
    srv.close()


def test_native_3d_step_equals_crm_run(gpu_lib):
    """The service with a 3D configuration (16 x 16 x 58, FP64): the first
    step of a chunk equals crm_run of the same columns bit for bit."""
    from crm_gb300.lib import CrmContext
    from crm_gb300.native_server import NativeCrmServer
    cfg, cin, st, rad, desc = S.workload_3d(ncrms=3, nx=16, ny=16, precision=T.CRM_FP64)
    gcol = list(np.asarray(desc._keep))
    dt_gl = 100.0
    srv = NativeCrmServer(cfg, capacity=8, handles=2)
    c = srv.open_chunk(st, rad, gcol)
    t = srv.submit(c, cin, 3, dt_gl, rad_means=True)
    assert t.poll() == 0 and not t.status.any()
    st_dev, _ = srv.read_state(c, 3)
    srv.close()
    c2 = T.CrmConfig(**{**cfg.__dict__, 'max_ncrms': 3})
    out = T.CrmOutput(3, cfg.crm_nx, cfg.crm_ny, cfg.crm_nz, cfg.plev)
    st2, rad2 = st.copy(), rad.copy()
    status = CrmContext(c2).run(T.call_desc(3, 3, dt_gl, 1, gcol), cin, st2, rad2, out)
    assert not status.any()
    for n, v in out.arrays().items():
        assert np.array_equal(v, getattr(t.out, n)), n
    for n, v in st2.arrays().items():
        assert np.array_equal(v, getattr(st_dev, n)), n
