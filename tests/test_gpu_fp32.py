"""FP32-mixed form against the FP64 oracle.

The mixed form keeps FP64 only for the pressure tridiagonal solve, the domain
sums and the saturation-adjustment Newton iteration; t and qt carry per-cell
FP32 residues of their updates, the projected w has its level means taken
out, and t is advected as an offset from a column constant.  After one GCM step (60-120 CRM steps of a
convecting boundary layer) rounding differences have been amplified by the
flow, so the comparison is statistical: relative L2 error per field, with the
bounds stated below, plus exact agreement of the status codes.
"""
import numpy as np
import pytest

import oracle
from crm_gb300 import synthetic as S
from crm_gb300 import crm_types as T
from crm_gb300.lib import CrmContext

from conftest import rel_l2

pytestmark = pytest.mark.gpu

# the tendency target: every GCM tendency within 1e-4 relative L2
TENDENCY_TARGET = 1e-4
# relative L2 bounds after one GCM step: state fields, and the GCM
# tendencies at the target; every other crm() output is held to
# OUTPUT_BOUND (measured <= 6e-3)
BOUNDS = {'temperature': 1e-6, 'qt': 2e-5, 'u_wind': 1e-4, 'w_wind': 3e-3, 'qp': 5e-4,
          'sltend': TENDENCY_TARGET, 'qltend': TENDENCY_TARGET, 'qcltend': TENDENCY_TARGET,
          'qiltend': TENDENCY_TARGET}
OUTPUT_BOUND = 3e-2


def _errors(wl, **kw):
    cfg, cin, st, rad, desc = wl(**kw)
    st_o, rad_o = st.copy(), rad.copy()
    rc, _, out_o = oracle.run(cfg, desc, cin, st_o, rad_o)
    assert rc == 0
    cfg.precision = T.CRM_FP32_MIXED
    cfg.max_ncrms = desc.ld
    ctx = CrmContext(cfg)
    out_g = T.CrmOutput(desc.ld, cfg.crm_nx, cfg.crm_ny, cfg.crm_nz, cfg.plev)
    st_g, rad_g = st.copy(), rad.copy()
    ctx.run(desc, cin, st_g, rad_g, out_g, raise_on_error=True)
    e = {n: rel_l2(getattr(st_g, n), getattr(st_o, n)) for n in ('temperature', 'qt', 'u_wind', 'w_wind', 'qp')}
    for n, a in out_g.arrays().items():
        assert np.isfinite(a).all(), n
        e[n] = rel_l2(a, getattr(out_o, n))
    return e


def _check(e, **override):
    for n, b in {**BOUNDS, **override}.items():
        assert e[n] <= b, (n, e[n], b)
    for n, v in e.items():
        assert v <= OUTPUT_BOUND, (n, v, OUTPUT_BOUND)


@pytest.mark.parametrize('moist', [False, True])
def test_fp32_mixed_32x28(gpu_lib, moist):
    e = _errors(S.workload_32x28, ncrms=4, moist=moist)
    print('fp32-mixed rel-L2 vs fp64 oracle (32x28, moist=%s):' % moist, e)
    _check(e)


@pytest.mark.parametrize('moist', [False, True])
def test_fp32_mixed_64x58(gpu_lib, moist):
    e = _errors(S.workload_64x58, ncrms=4, moist=moist)
    print('fp32-mixed rel-L2 vs fp64 oracle (64x58, moist=%s):' % moist, e)
    _check(e)


def test_fp32_mixed_mean_state_acceleration(gpu_lib):
    def wl(**kw):
        cfg, cin, st, rad, desc = S.workload_32x28(**kw)
        cfg = T.CrmConfig(**{**cfg.__dict__, 'use_crm_accel': 1, 'crm_accel_factor': 2.0})
        return cfg, cin, st, rad, desc
    e = _errors(wl, ncrms=4, moist=True)
    print('fp32-mixed rel-L2 vs fp64 oracle (32x28, accelerated):', e)
    # the acceleration multiplies each level mean's change per step, and its
    # rounding, by up to 1 + crm_accel_factor = 3: the target scaled by 3
    _check(e, **{n: 3 * TENDENCY_TARGET for n in ('sltend', 'qltend', 'qcltend', 'qiltend')})


def test_fp32_mixed_water_budget(gpu_lib):
    """Column water change = large-scale forcing - surface precipitation: the
    FP64 oracle closes it to ~1e-16 relative; the FP32-mixed form (state kept
    in FP32) to the FP32 rounding of the column water."""
    from test_oracle import water_residual
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=4, moist=True)
    cfg.precision = T.CRM_FP32_MIXED
    cfg.max_ncrms = 4
    ctx = CrmContext(cfg)
    out = T.CrmOutput(4, cfg.crm_nx, 1, cfg.crm_nz, cfg.plev)
    st1 = st.copy()
    ctx.run(desc, cin, st1, rad.copy(), out, raise_on_error=True)
    r = water_residual(cfg, cin, st, st1, out, desc.dt_gl)
    print('fp32-mixed column water residual (relative):', r)
    assert np.max(np.abs(r)) < 1e-5, r


def test_fp32_mixed_gcm_water_identity(gpu_lib):
    """The GCM-side identity of check_energy_chng (column water tendency +
    surface precipitation + CRM precipitation storage = 0) for the FP32-mixed
    form: its tendencies are FP64 sums of FP32 fields, so the identity holds
    to the FP32 rounding of the CRM state."""
    from crm_gb300 import gcm_coupling as G
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=4, moist=True)
    cfg.precision = T.CRM_FP32_MIXED
    cfg.max_ncrms = 4
    ctx = CrmContext(cfg)
    out = T.CrmOutput(4, cfg.crm_nx, 1, cfg.crm_nz, cfg.plev)
    ctx.run(desc, cin, st.copy(), rad.copy(), out, raise_on_error=True)
    r = G.water_residual(cin, out, 4) / G.water_scale(cin, out, 4)
    print('fp32-mixed GCM water identity residual (relative):', r)
    assert np.max(np.abs(r)) < 1e-4, r


@pytest.mark.parametrize('moist', [False, True])
def test_fp32_mixed_gcm_energy_identity(gpu_lib, moist):
    """The column energy identity (energy tendency = radiative heating +
    latent heat of the surface precipitation and of the CRM's precipitation
    storage change) for the FP32-mixed form; the FP64 oracle closes it to
    ~1e-8 of its terms."""
    from crm_gb300 import gcm_coupling as G
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=4, moist=moist)
    cfg.precision = T.CRM_FP32_MIXED
    cfg.max_ncrms = 4
    ctx = CrmContext(cfg)
    out = T.CrmOutput(4, cfg.crm_nx, 1, cfg.crm_nz, cfg.plev)
    rad_in = rad.copy()
    ctx.run(desc, cin, st.copy(), rad.copy(), out, raise_on_error=True)
    r = G.energy_residual(cin, rad_in, out, 4, cfg.crm_nz) / G.energy_scale(cin, rad_in, out, 4, cfg.crm_nz)
    print('fp32-mixed GCM energy identity residual (relative, moist=%s):' % moist, r)
    assert np.max(np.abs(r)) < 1e-3, r


def test_fp32_mixed_reference_batch_mode(gpu_lib):
    """CRM_REFERENCE_BATCH in the FP32-mixed form: the grid-wide maxima
    couple the columns the same way (ncycle from the batch), within the
    FP32 bounds of the oracle's batch mode."""
    def wl(**kw):
        cfg, cin, st, rad, desc = S.workload_32x28(**kw)
        cfg = T.CrmConfig(**{**cfg.__dict__, 'batch_mode': T.CRM_REFERENCE_BATCH})
        desc.dt_gl = 400.0
        st.w_wind[2, :, :, 10] = 40.0
        return cfg, cin, st, rad, desc
    e = _errors(wl, ncrms=4, moist=True)
    print('fp32-mixed rel-L2 vs fp64 oracle (32x28, reference batch mode):', e)
    # a 40 m/s column drives the batch's ncycle: ten times the field bounds,
    # 5e-3 on the tendencies
    for n, b in (('temperature', 1e-5), ('qt', 2e-4), ('u_wind', 1e-3), ('sltend', 5e-3), ('qltend', 5e-3)):
        assert e[n] <= b, (n, e[n])


@pytest.mark.parametrize('moist', [False, True])
def test_fp32_mixed_w_has_zero_level_means(gpu_lib, moist):
    """The projected w has zero horizontal mean at every level in exact
    arithmetic (anelastic continuity, periodic sides, w = 0 at the surface);
    the FP32-mixed form takes the FP32 rounding of that mean out of the new
    w each substep, so the returned state's level means sit at the rounding
    of the subtraction, not at the ~1e-6 of the rms that the FP32 momentum
    and pressure phases leave."""
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=4, moist=moist)
    cfg.precision = T.CRM_FP32_MIXED
    cfg.max_ncrms = desc.ld
    out = T.CrmOutput(desc.ld, cfg.crm_nx, cfg.crm_ny, cfg.crm_nz, cfg.plev)
    CrmContext(cfg).run(desc, cin, st, rad, out, raise_on_error=True)
    w = st.w_wind[:4].reshape(4, cfg.crm_nx, cfg.crm_nz)        # (column, x, level)
    rms = np.sqrt((w[:, :, 1:] ** 2).mean(axis=1))
    mean = np.abs(w[:, :, 1:].mean(axis=1))
    rel = np.where(rms > 0, mean / np.maximum(rms, 1e-30), 0.0)
    print('FP32-mixed largest |level mean of w| / rms (moist=%s): %.2e' % (moist, rel.max()))
    assert rel.max() <= 1e-7, rel.max()
