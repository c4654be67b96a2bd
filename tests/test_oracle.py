"""CPU checks of the oracle (the FP64 restatement of crm()).

The reference ships no golden vectors for crm(), so these checks pin the
restatement by properties the reference's algorithm has:

  * the column water budget closes: the change of column water (qt + qp,
    weighted by pdel/g) equals the large-scale forcing minus surface
    precipitation, to rounding (flux-form MPDATA and sedimentation with
    closed top and bottom, mass-conserving negative-water fixer);
  * the periodic domain is translation invariant: rolling the initial state
    in x rolls the result (to rounding in the FFT);
  * a horizontally uniform state stays uniform;
  * per-column mode makes every column independent of its batch mates, and
    equals the reference's batch coupling when no column sub-cycles;
  * the OpenMP thread count does not change a bit;
  * a column that breaks the CFL limit is flagged without touching the rest.
"""
import numpy as np
import pytest

import oracle
from crm_gb300 import crm_types as T
from crm_gb300 import synthetic as S

GRAV = 9.80616


def _run(cfg, cin, st, rad, desc, nthreads=0):
    st, rad = st.copy(), rad.copy()
    rc, stat, out = oracle.run(cfg, desc, cin, st, rad, nthreads=nthreads)
    return rc, stat, st, rad, out


def _equal(a, b):
    """Names of the fields of (state, rad, out) that differ."""
    bad = []
    for x, y, tag in ((a[0], b[0], 'state'), (a[1], b[1], 'rad'), (a[2], b[2], 'out')):
        for n, v in x.arrays().items():
            if not np.array_equal(v, getattr(y, n)):
                bad.append(tag + '.' + n)
    return bad


def water_residual(cfg, cin, st0, st1, out, dt_gl):
    """Per column: (dW - forcing + P) / W0 with W the pdel/g-weighted column water."""
    nz, plev = cfg.crm_nz, cfg.plev
    res = []
    for c in range(st0.qt.shape[0]):
        pd = np.array([cin.pdel[c, plev - 1 - k] for k in range(nz)]) / GRAV
        w0 = np.sum(pd * (st0.qt[c, :, 0, :] + st0.qp[c, :, 0, :]).mean(axis=0))
        w1 = np.sum(pd * (st1.qt[c, :, 0, :] + st1.qp[c, :, 0, :]).mean(axis=0))
        forc = np.sum(pd * np.array([out.qt_ls[c, plev - 1 - k] for k in range(nz)])) * dt_gl
        prec = (out.precc[c] + out.precl[c]) * 1000.0 * dt_gl
        res.append((w1 - w0 - forc + prec) / w0)
    return np.array(res)


@pytest.mark.parametrize('moist', [False, True])
def test_water_budget_closes_32x28(moist):
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=4, moist=moist)
    rc, stat, st1, _, out = _run(cfg, cin, st, rad, desc)
    assert rc == 0 and not stat.any()
    r = water_residual(cfg, cin, st, st1, out, desc.dt_gl)
    assert np.max(np.abs(r)) < 1e-13, r
    if moist:
        assert np.all(out.precc + out.precl > 0)


def test_water_budget_closes_64x58():
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=2, moist=True)
    desc.dt_gl = 300.0
    rc, stat, st1, _, out = _run(cfg, cin, st, rad, desc)
    assert rc == 0 and not stat.any()
    r = water_residual(cfg, cin, st, st1, out, desc.dt_gl)
    assert np.max(np.abs(r)) < 1e-13, r


def test_thread_count_does_not_change_results():
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=6, moist=True)
    desc.dt_gl = 400.0
    a = _run(cfg, cin, st, rad, desc, nthreads=1)
    b = _run(cfg, cin, st, rad, desc, nthreads=3)
    assert not _equal(a[2:], b[2:])


def test_columns_independent_of_batch_mates():
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=6, moist=True)
    desc.dt_gl = 400.0
    full = _run(cfg, cin, st, rad, desc)
    gcol = np.asarray(desc._keep)
    for cols in ([0, 1, 2], [5, 3]):
        d = T.call_desc(len(cols), len(cols), desc.dt_gl, desc.igstep, gcol[cols])
        part = _run(cfg, cin.take(cols), st.take(cols), rad.take(cols), d)
        ref = (full[2].take(cols), full[3].take(cols))
        for n, v in ref[0].arrays().items():
            assert np.array_equal(v, getattr(part[2], n)), n
        for n, v in part[4].arrays().items():
            assert np.array_equal(v, getattr(full[4], n)[cols]), n


def test_reference_batch_mode_equals_per_column_without_subcycling():
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=4, moist=True)
    desc.dt_gl = 400.0
    a = _run(cfg, cin, st, rad, desc)
    cfg_b = S.config_32x28(batch_mode=T.CRM_REFERENCE_BATCH)
    b = _run(cfg_b, cin, st, rad, desc)
    assert a[0] == 0 and b[0] == 0
    assert not _equal(a[2:], b[2:])


def test_translation_invariance():
    # The reference's fft991 builds its twiddles in REAL*4 (implicit typing in
    # fft.F90), so forward and inverse transforms are exact inverses, and
    # shift-equivariant, only to ~1e-7 relative: a shifted run differs at that
    # level in the pressure correction.  An indexing or halo error would show
    # as an O(1) difference of the perturbation fields.
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=2)
    d = T.call_desc(2, 2, 100.0, 2, desc._keep)     # igstep 2: no setperturb
    a = _run(cfg, cin, st, rad, d)
    sh = 5
    st_r = st.copy()
    for n, v in st_r.arrays().items():
        v[...] = np.roll(v, sh, axis=1)
    b = _run(cfg, cin, st_r, rad, d)
    for n, v in a[2].arrays().items():
        x = np.roll(v, sh, axis=1)
        y = getattr(b[2], n)
        spread = np.max(np.abs(v - v.mean(axis=1, keepdims=True)))
        if spread == 0.0:
            assert np.array_equal(x, y), n
            continue
        assert np.max(np.abs(x - y)) <= 1e-4 * spread, (n, np.max(np.abs(x - y)), spread)
    for n in ('sltend', 'qltend'):
        x, y = getattr(a[4], n), getattr(b[4], n)
        assert np.max(np.abs(x - y)) <= 1e-4 * (np.max(np.abs(x)) or 1.0), n


def test_uniform_state_stays_uniform():
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=2)
    st.temperature[...] = st.temperature[:, :1]     # drop the seeded perturbation
    d = T.call_desc(2, 2, 400.0, 2, desc._keep)     # and setperturb
    _, stat, st1, _, _ = _run(cfg, cin, st, rad, d)
    assert not stat.any()
    for n, v in st1.arrays().items():
        spread = np.max(np.abs(v - v[:, :1]))
        assert spread <= 1e-10 * (np.max(np.abs(v)) or 1.0), (n, spread)


def test_cfl_violation_flags_only_that_column():
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=3)
    desc.dt_gl = 100.0
    st.w_wind[1, :, :, 10] = 2000.0
    rc, stat, st1, _, out = _run(cfg, cin, st, rad, desc)
    assert list(stat) == [0, T.CRM_ERR_CFL, 0]
    assert rc == T.CRM_ERR_CFL
    ok = _run(cfg, cin.take([0, 2]), st.take([0, 2]), rad.take([0, 2]),
              T.call_desc(2, 2, 100.0, desc.igstep, np.asarray(desc._keep)[[0, 2]]))
    for n, v in ok[2].arrays().items():
        assert np.array_equal(v, getattr(st1, n)[[0, 2]]), n


def test_col_map_selects_slots():
    """A call over slots (3, 0) of a 5-column batch equals a call over a
    2-column batch holding those columns; other slots are untouched."""
    import ctypes as C
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=5, moist=True)
    gcol = np.asarray(desc._keep)
    slots = np.array([3, 0], dtype=np.int32)
    d = T.call_desc(2, 5, 400.0, desc.igstep, gcol[slots])
    d.col_map = slots.ctypes.data_as(C.POINTER(C.c_int))
    a = _run(cfg, cin, st, rad, d)
    assert a[0] == 0
    b = _run(cfg, cin.take(slots), st.take(slots), rad.take(slots),
             T.call_desc(2, 2, 400.0, desc.igstep, gcol[slots]))
    for n, v in b[2].arrays().items():
        assert np.array_equal(getattr(a[2], n)[slots], v), n
        untouched = [1, 2, 4]
        assert np.array_equal(getattr(a[2], n)[untouched], getattr(st, n)[untouched]), n
    for n, v in b[4].arrays().items():
        assert np.array_equal(getattr(a[4], n)[slots], v), n


def _accel(cfg, factor=2.0, uv=0):
    return T.CrmConfig(**{**cfg.__dict__, 'use_crm_accel': 1, 'crm_accel_factor': factor,
                          'crm_accel_uv': uv})


def test_accel_requires_dividing_factor():
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=2)
    desc.dt_gl = 200.0                       # nstop 10: 1 + 2 does not divide it
    rc, _, _ = oracle.run(_accel(cfg, 2.0), desc, cin, st.copy(), rad.copy())
    assert rc == T.CRM_ERR_ARG
    rc, _, _ = oracle.run(_accel(cfg, 1.0), desc, cin, st.copy(), rad.copy())
    assert rc == 0


@pytest.mark.parametrize('uv', [0, 1])
def test_accel_changes_mean_state_and_matches_batch_mode(uv):
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=3, moist=True)
    desc.dt_gl = 600.0                       # 30 steps -> 10 accelerated steps
    plain = _run(cfg, cin, st, rad, desc)
    acc = _run(_accel(cfg, 2.0, uv), cin, st, rad, desc)
    assert acc[0] == 0
    for n, v in acc[2].arrays().items():
        assert np.all(np.isfinite(v)), n
    assert not np.array_equal(acc[2].temperature, plain[2].temperature)
    bcfg = _accel(S.config_32x28(batch_mode=T.CRM_REFERENCE_BATCH), 2.0, uv)
    batch = _run(bcfg, cin, st, rad, desc)
    assert batch[0] == 0
    assert not _equal(acc[2:], batch[2:])


def test_accel_ceases_on_large_mean_temperature_change():
    """A column heated by ~10 K per step trips the 5 K limit: acceleration
    stops and the remaining steps run unaccelerated (nstop stretched)."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=2)
    desc.dt_gl = 600.0
    rad_hot = rad.copy()
    rad_hot.qrad[1, :, :, 5:8] = 0.5         # K/s in column 1 only
    acc = _run(_accel(cfg, 2.0), cin, st, rad_hot, desc)
    assert acc[0] == 0
    # column 0 is unaffected by column 1's cease (per-column mode)
    alone = _run(_accel(cfg, 2.0), cin.take([0]), st.take([0]), rad_hot.take([0]),
                 T.call_desc(1, 1, 600.0, desc.igstep, np.asarray(desc._keep)[[0]]))
    for n, v in alone[2].arrays().items():
        assert np.array_equal(v[0], getattr(acc[2], n)[0]), n
    # column 1 ceases at its first step, before any acceleration is applied,
    # and its nstop grows from 10 to 10 + 10 * 2 = 30: exactly the plain run
    plain = _run(cfg, cin, st, rad_hot, desc)
    for n, v in plain[2].arrays().items():
        assert np.array_equal(v[1], getattr(acc[2], n)[1]), n
    for n, v in plain[4].arrays().items():
        assert np.array_equal(v[1], getattr(acc[4], n)[1]), n


def test_nonfinite_column_is_reported_and_isolated():
    """A NaN in one column's state stops that column with CRM_ERR_NONFINITE
    (the reference has no such check and carries the NaN on); the other
    columns give the same bits as a batch without it."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=3)
    desc.dt_gl = 200.0
    bad = st.copy()
    bad.temperature[1, 7, 0, 2] = np.nan
    rc, stat, st_b, rad_b, out_b = _run(cfg, cin, bad, rad, desc)
    assert rc == T.CRM_ERR_NONFINITE and list(stat) == [0, T.CRM_ERR_NONFINITE, 0]
    rc, stat, st_g, rad_g, out_g = _run(cfg, cin, st, rad, desc)
    assert rc == 0
    for x, y in ((st_b, st_g), (rad_b, rad_g), (out_b, out_g)):
        for n, v in x.arrays().items():
            w = getattr(y, n)
            assert np.array_equal(v[[0, 2]], w[[0, 2]]), n


def test_nonfinite_column_stops_a_reference_batch():
    """Batch mode: the non-finite column's unbounded CFL stops the batch;
    it reports CRM_ERR_NONFINITE and the others CRM_ERR_CFL."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=3, batch_mode=T.CRM_REFERENCE_BATCH)
    desc.dt_gl = 200.0
    st.w_wind[2, 3, 0, 5] = np.inf
    rc, stat, *_ = _run(cfg, cin, st, rad, desc)
    assert list(stat) == [T.CRM_ERR_CFL, T.CRM_ERR_CFL, T.CRM_ERR_NONFINITE]
