"""FP64 device form against the CPU restatement, through the C ABI.

Both evaluate the same IEEE operations in the same order (no FMA contraction,
deterministic exp/log/pow, horizontal sums in the reference's loop order), so
every state, rad and output field must agree bit for bit: the tolerance of
these tests is zero.
"""
import numpy as np
import pytest

import oracle
from crm_gb300 import synthetic as S
from crm_gb300 import crm_types as T
from crm_gb300.lib import CrmContext

pytestmark = pytest.mark.gpu

_ctx = {}


def _context(cfg):
    key = tuple(sorted(cfg.__dict__.items()))
    if key not in _ctx:
        _ctx[key] = CrmContext(cfg)
    return _ctx[key]


def run_gpu(cfg, cin, st, rad, desc):
    cfg.max_ncrms = max(cfg.max_ncrms, desc.ld)
    ctx = _context(cfg)
    out = T.CrmOutput(desc.ld, cfg.crm_nx, cfg.crm_ny, cfg.crm_nz, cfg.plev)
    stat = ctx.run(desc, cin, st, rad, out)
    return ctx.last_rc, stat, out


def run_both(cfg, cin, st, rad, desc):
    st_o, rad_o = st.copy(), rad.copy()
    rc, stat_o, out_o = oracle.run(cfg, desc, cin, st_o, rad_o)
    assert rc == 0, stat_o
    st_g, rad_g = st.copy(), rad.copy()
    rc_g, stat_g, out_g = run_gpu(cfg, cin, st_g, rad_g, desc)
    assert rc_g == 0, stat_g
    return (st_o, rad_o, out_o), (st_g, rad_g, out_g)


def mismatches(a, b):
    (st_o, rad_o, out_o), (st_g, rad_g, out_g) = a, b
    bad = []
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


def test_fp64_bitexact_32x28_short(gpu_lib):
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=4)
    desc.dt_gl = 200.0          # 10 CRM steps
    assert mismatches(*run_both(cfg, cin, st, rad, desc)) == []


def test_fp64_bitexact_32x28_full(gpu_lib):
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=16)
    assert mismatches(*run_both(cfg, cin, st, rad, desc)) == []


def test_fp64_bitexact_32x28_moist(gpu_lib):
    """Supersaturated layers, falling rain and ice: every microphysics branch."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=4, moist=True)
    a, b = run_both(cfg, cin, st, rad, desc)
    assert a[2].cltot.max() > 0 and a[2].precc.max() > 0
    assert mismatches(a, b) == []


def test_fp64_bitexact_64x58(gpu_lib):
    """64 x 58 columns, dx 1 km, 120 CRM steps."""
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=4)
    assert mismatches(*run_both(cfg, cin, st, rad, desc)) == []


def test_fp64_bitexact_64x58_moist(gpu_lib):
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=2, moist=True)
    assert mismatches(*run_both(cfg, cin, st, rad, desc)) == []


@pytest.mark.parametrize('nx', [16, 128])
def test_fp64_bitexact_other_nx(gpu_lib, nx):
    """nx = 128 (a compile-time size) and nx = 16 (the generic kernel)."""
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=2, nx=nx, moist=True)
    desc.dt_gl = 300.0
    assert mismatches(*run_both(cfg, cin, st, rad, desc)) == []


def test_fp64_bitexact_three_gcm_steps(gpu_lib):
    """State carried across three calls (igstep 1, 2, 3), as in a GCM run."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=3, moist=True)
    st_o, rad_o, st_g, rad_g = st.copy(), rad.copy(), st.copy(), rad.copy()
    for step in (1, 2, 3):
        desc.igstep = step
        rc, _, out_o = oracle.run(cfg, desc, cin, st_o, rad_o)
        assert rc == 0
        rc, _, out_g = run_gpu(cfg, cin, st_g, rad_g, desc)
        assert rc == 0
        assert mismatches((st_o, rad_o, out_o), (st_g, rad_g, out_g)) == [], step


def test_columns_independent_and_ld_padding(gpu_lib):
    """Per-column mode: a column's result is the same alone and in a batch,
    and columns beyond ncrms of a padded (ld > ncrms) array are untouched."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=5, moist=True)
    st_all = st.copy()
    rad_all = rad.copy()
    rc, _, out_all = run_gpu(cfg, cin, st_all, rad_all, desc)
    assert rc == 0
    # column 3 alone, inside an ld = 5 array with ncrms = 1 after moving it to slot 0
    cin1, st1, rad1 = cin.copy(), st.copy(), rad.copy()
    for b in (cin1, st1, rad1):
        for n, a in b.arrays().items():
            a[0] = a[3]
    d1 = T.call_desc(1, desc.ld, desc.dt_gl, desc.igstep, [4, 0, 0, 0, 0])
    before = st1.temperature[1:].copy()
    rc, _, out1 = run_gpu(cfg, cin1, st1, rad1, d1)
    assert rc == 0
    assert np.array_equal(st1.temperature[1:], before)
    for n, a in st_all.arrays().items():
        assert np.array_equal(a[3], getattr(st1, n)[0]), n
    for n, a in out_all.arrays().items():
        assert np.array_equal(a[3], getattr(out1, n)[0]), n


def test_cfl_violation_is_reported_per_column(gpu_lib):
    """kurant() needs > 16 subcycles: the reference aborts the model
    (kurant.F90:66-75); here only that column reports CRM_ERR_CFL."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=3)
    st.w_wind[1, 5, 0, 3] = 400.0
    st_o = st.copy()
    rc_o, stat_o, _ = oracle.run(cfg, desc, cin, st_o, rad.copy())
    rc, stat, _ = run_gpu(cfg, cin, st.copy(), rad.copy(), desc)
    assert rc == T.CRM_ERR_CFL and rc_o == T.CRM_ERR_CFL
    assert list(stat) == [0, T.CRM_ERR_CFL, 0]
    assert list(stat_o) == [0, T.CRM_ERR_CFL, 0]


def test_device_path_matches_host_path(gpu_lib):
    """crm_run_device on device-resident arrays == crm_run on host arrays."""
    import torch
    from crm_gb300.device import DeviceCrmArrays
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=4, moist=True)
    st_h, rad_h = st.copy(), rad.copy()
    rc, _, out_h = run_gpu(cfg, cin, st_h, rad_h, desc)
    assert rc == 0
    ctx = _context(cfg)
    dev = DeviceCrmArrays(cfg, cin, st, rad, desc, desc._keep)
    ctx.run_device(dev, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for n in T.STATE_FIELDS:
        assert np.array_equal(dev.state_numpy(n), getattr(st_h, n)), n
    for n, _ in T.OUTPUT_FIELDS:
        assert np.array_equal(dev.out_numpy(n), getattr(out_h, n)), n
    assert int(dev.status.sum().item()) == 0


def test_col_map_matches_oracle(gpu_lib):
    """A call over slots (3, 0, 4) of a 5-column batch (col_map), bit for bit
    against the oracle given the same map."""
    import ctypes as C
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=5, moist=True)
    slots = np.array([3, 0, 4], dtype=np.int32)
    d = T.call_desc(3, 5, 400.0, desc.igstep, np.asarray(desc._keep)[slots])
    d.col_map = slots.ctypes.data_as(C.POINTER(C.c_int))
    a, b = run_both(cfg, cin, st, rad, d)
    assert mismatches(a, b) == []
    assert np.array_equal(b[0].temperature[[1, 2]], st.temperature[[1, 2]])


def _accel(cfg, factor=2.0, uv=0):
    return T.CrmConfig(**{**cfg.__dict__, 'use_crm_accel': 1, 'crm_accel_factor': factor,
                          'crm_accel_uv': uv})


@pytest.mark.parametrize('uv', [0, 1])
def test_fp64_bitexact_mean_state_acceleration(gpu_lib, uv):
    """use_crm_accel with crm_accel_factor 2 (the sam1mom production default),
    with and without crm_accel_uv."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=4, moist=True)
    desc.dt_gl = 600.0
    assert mismatches(*run_both(_accel(cfg, 2.0, uv), cin, st, rad, desc)) == []


def test_fp64_bitexact_acceleration_cease(gpu_lib):
    """A column heated ~10 K per step stops accelerating (nstop stretched);
    its batch mate keeps accelerating."""
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=2, moist=True)
    desc.dt_gl = 300.0
    rad.qrad[1, :, :, 5:8] = 1.0
    assert mismatches(*run_both(_accel(cfg, 2.0), cin, st, rad, desc)) == []


def test_fp64_bitexact_reference_batch_mode(gpu_lib):
    """CRM_REFERENCE_BATCH on the GPU (one cooperative launch, grid-wide
    maxima): one column strong enough to need sub-cycling sets ncycle for the
    whole batch, bit for bit as the oracle's batch mode does."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=4, moist=True)
    desc.dt_gl = 400.0
    st.w_wind[2, :, :, 10] = 40.0
    bcfg = S.config_32x28(batch_mode=T.CRM_REFERENCE_BATCH)
    a, b = run_both(bcfg, cin, st, rad, desc)
    assert mismatches(a, b) == []
    # the coupling is real: per-column mode gives the other columns other bits
    pc, _ = run_both(cfg, cin, st, rad, desc)
    assert not np.array_equal(pc[0].temperature[0], a[0].temperature[0])
    assert np.array_equal(pc[0].temperature[2], a[0].temperature[2])


def test_fp64_bitexact_reference_batch_acceleration_cease(gpu_lib):
    """Batch mode with mean-state acceleration: one hot column stops the
    acceleration of every column (one cease flag per batch)."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=3)
    desc.dt_gl = 600.0
    rad.qrad[1, :, :, 5:8] = 0.5
    bcfg = _accel(S.config_32x28(batch_mode=T.CRM_REFERENCE_BATCH), 2.0)
    assert mismatches(*run_both(bcfg, cin, st, rad, desc)) == []


def test_fp64_bitexact_mixed_precipitating_columns(gpu_lib):
    """Columns with and without precipitating water in one batch: the kernel
    skips sedimentation and qp transport for a column whose fall speeds are
    all zero or whose qp is +0 everywhere, which must change no bit — signs
    of zero included — of any column's state or outputs."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=6, moist=True)
    _, cin_d, st_d, _, _ = S.workload_32x28(ncrms=6, moist=False)
    for c in (1, 3, 5):                       # dry columns between moist ones
        for n in ('qt', 'qp', 'qn', 'temperature'):
            getattr(st, n)[c] = getattr(st_d, n)[c]
        cin.qccl[c] = cin_d.qccl[c]
        cin.qiil[c] = cin_d.qiil[c]
    a, b = run_both(cfg, cin, st, rad, desc)
    assert mismatches(a, b) == []
    (st_o, _, out_o), (st_g, _, out_g) = a, b
    assert np.any(st_o.qp[0] > 0) and not np.any(st_o.qp[1] > 0)
    for n, x in list(st_o.arrays().items()) + list(out_o.arrays().items()):
        y = getattr(st_g, n) if n in st_o.arrays() else getattr(out_g, n)
        xb = np.ascontiguousarray(x).view(np.uint64)
        yb = np.ascontiguousarray(y).view(np.uint64)
        assert np.array_equal(xb, yb), n


def test_col_map_slot_out_of_range_is_reported_per_column(gpu_lib):
    """A col_map entry outside 0..ld-1 is refused by the set-up and column
    kernels before they touch that slot: its position reports
    CRM_ERR_ARG, the other positions integrate as in a call without it."""
    import ctypes as C
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=5, moist=True)
    desc.dt_gl = 200.0
    keep = np.asarray(desc._keep)
    good = np.array([3, 0], dtype=np.int32)
    bad = np.array([3, 5, 0, -1], dtype=np.int32)       # 5 = ld, -1: out of range
    d_good = T.call_desc(2, 5, desc.dt_gl, desc.igstep, keep[good])
    d_good.col_map = good.ctypes.data_as(C.POINTER(C.c_int))
    gcol_bad = np.array([keep[3], keep[0], keep[0], keep[0]], dtype=np.int32)
    d_bad = T.call_desc(4, 5, desc.dt_gl, desc.igstep, gcol_bad)
    d_bad.col_map = bad.ctypes.data_as(C.POINTER(C.c_int))
    st_a, rad_a = st.copy(), rad.copy()
    rc_a, stat_a, out_a = run_gpu(cfg, cin, st_a, rad_a, d_good)
    assert rc_a == 0, stat_a
    st_b, rad_b = st.copy(), rad.copy()
    rc_b, stat_b, out_b = run_gpu(cfg, cin, st_b, rad_b, d_bad)
    assert list(stat_b) == [T.CRM_OK, T.CRM_ERR_ARG, T.CRM_OK, T.CRM_ERR_ARG], stat_b
    assert rc_b == T.CRM_ERR_ARG
    for n, x in st_a.arrays().items():
        assert np.array_equal(x, getattr(st_b, n)), n
    for n, x in out_a.arrays().items():
        assert np.array_equal(x[[3, 0]], getattr(out_b, n)[[3, 0]]), n


@pytest.mark.parametrize('seed', range(4))
def test_fp64_bitexact_random_columns(gpu_lib, seed):
    """Random soundings, surface fluxes, winds, moisture and call lengths
    (the cases of test_oracle_properties.py): bit for bit."""
    from test_oracle_properties import _case
    cfg, cin, st, rad, desc, ncol = _case(seed)
    assert mismatches(*run_both(cfg, cin, st, rad, desc)) == []


@pytest.mark.parametrize('nx', [48, 80])
def test_fp64_bitexact_radix_3_and_5_sizes(gpu_lib, nx):
    """crm_nx with transform factors 3 (48 = 2 x 3 x 8) and 5 (80 = 2 x 5 x 8):
    the warp FFT's radix-3 and radix-5 passes (fft.F90 vpassm_crm)."""
    base = S.config_32x28()
    cfg = T.CrmConfig(**{**base.__dict__, 'crm_nx': nx, 'crm_nx_rad': nx})
    cin, st, rad, desc = S.make_inputs(cfg, 3, 300.0, 10.0, 100.0, seed=nx, moist=True)
    desc.dt_gl = 400.0
    assert mismatches(*run_both(cfg, cin, st, rad, desc)) == []

