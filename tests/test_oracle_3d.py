"""The oracle's 3D CRM (crm_ny > 1): advect_scalar3D, diffuse_mom3D,
diffuse_scalar3D, shear_prod3D, the y terms of advect2_mom_xy/z and the
2D x/y transform of the pressure solve.

The reference ships no 3D outputs to compare with, so these check what the
3D discretisation must satisfy:
  * the column water budget closes (MPDATA and the SGS fluxes conserve);
  * a horizontally uniform state stays uniform;
  * a state shifted in x and in y gives shifted results (periodic halos);
  * the x-y transpose of a state with u <-> v gives the transpose of the
    results to round-off: the x and y code paths agree.
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


def _small(ncrms=2, nx=16, ny=16, nz=58, **kw):
    return S.workload_3d(ncrms=ncrms, nx=nx, ny=ny, nz=nz, **kw)


def test_3d_runs_and_moves_in_y():
    cfg, cin, st, rad, desc = _small()
    desc.dt_gl = 200.0
    rc, stat, st1, _, out = _run(cfg, cin, st, rad, desc)
    assert rc == 0 and not stat.any()
    for n, v in st1.arrays().items():
        assert np.all(np.isfinite(v)), n
    # v is a prognostic variable in 3D (it is zero in 2D) and varies in y
    assert np.max(np.abs(st1.v_wind)) > 1.0
    assert np.max(np.abs(st1.v_wind - st1.v_wind.mean(axis=2, keepdims=True))) > 1e-4


@pytest.mark.parametrize('moist', [False, True])
def test_3d_water_budget_closes(moist):
    cfg, cin, st, rad, desc = _small(moist=moist)
    desc.dt_gl = 600.0 if moist else 200.0     # rain from 2 km reaches the ground
    rc, stat, st1, _, out = _run(cfg, cin, st, rad, desc)
    assert rc == 0 and not stat.any()
    nz, plev = cfg.crm_nz, cfg.plev
    for c in range(2):
        pd = np.array([cin.pdel[c, plev - 1 - k] for k in range(nz)]) / GRAV
        w0 = np.sum(pd * (st.qt[c] + st.qp[c]).mean(axis=(0, 1)))
        w1 = np.sum(pd * (st1.qt[c] + st1.qp[c]).mean(axis=(0, 1)))
        forc = np.sum(pd * np.array([out.qt_ls[c, plev - 1 - k] for k in range(nz)])) * desc.dt_gl
        prec = (out.precc[c] + out.precl[c]) * 1000.0 * desc.dt_gl
        assert abs((w1 - w0 - forc + prec) / w0) < 1e-13
    if moist:
        assert np.all(out.precc + out.precl > 0)


def test_3d_uniform_state_stays_uniform():
    cfg, cin, st, rad, desc = _small()
    st.temperature[...] = st.temperature[:, :1, :1]
    d = T.call_desc(2, 2, 200.0, 2, desc._keep)          # igstep 2: no setperturb
    _, stat, st1, _, _ = _run(cfg, cin, st, rad, d)
    assert not stat.any()
    for n, v in st1.arrays().items():
        spread = np.max(np.abs(v - v[:, :1, :1]))
        assert spread <= 1e-10 * (np.max(np.abs(v)) or 1.0), (n, spread)


def _compare(a, b, tol=1e-4):
    for n, x in a.items():
        y = b[n]
        spread = np.max(np.abs(x - x.mean(axis=(1, 2), keepdims=True)))
        if spread == 0.0:
            assert np.max(np.abs(x - y)) <= 1e-12 * (np.max(np.abs(x)) or 1.0), n
            continue
        assert np.max(np.abs(x - y)) <= tol * spread, (n, np.max(np.abs(x - y)), spread)


def test_3d_translation_invariance():
    cfg, cin, st, rad, desc = _small()
    d = T.call_desc(2, 2, 100.0, 2, desc._keep)
    a = _run(cfg, cin, st, rad, d)
    sx, sy = 5, 3
    st_r = st.copy()
    for n, v in st_r.arrays().items():
        v[...] = np.roll(np.roll(v, sx, axis=1), sy, axis=2)
    b = _run(cfg, cin, st_r, rad, d)
    _compare({n: np.roll(np.roll(v, sx, axis=1), sy, axis=2) for n, v in a[2].arrays().items()},
             b[2].arrays())


def test_3d_transpose_symmetry():
    """x <-> y with u <-> v: the y code paths mirror the x ones."""
    cfg, cin, st, rad, desc = _small()
    cin = cin.copy()
    cin.vl[...] = cin.ul                  # the same mean wind along x and y
    st.v_wind[...] = st.u_wind
    # a perturbation symmetric under the transpose, no setperturb
    t = st.temperature
    t[...] = 0.5 * (t + t.transpose(0, 2, 1, 3))
    d = T.call_desc(2, 2, 100.0, 2, desc._keep)
    a = _run(cfg, cin, st, rad, d)
    st_t = st.copy()
    for n, v in st_t.arrays().items():
        v[...] = getattr(st, n).transpose(0, 2, 1, 3)
    st_t.u_wind[...], st_t.v_wind[...] = st.v_wind.transpose(0, 2, 1, 3), st.u_wind.transpose(0, 2, 1, 3)
    b = _run(cfg, cin, st_t, rad, d)
    x = {n: v.transpose(0, 2, 1, 3) for n, v in a[2].arrays().items()}
    x['u_wind'], x['v_wind'] = a[2].v_wind.transpose(0, 2, 1, 3), a[2].u_wind.transpose(0, 2, 1, 3)
    # u(i) sits at the west face of cell i and v(j) at its south face, so the
    # transpose maps faces to faces; the two runs differ only by the order of
    # the x and y transforms (measured: 1e-12 of the perturbations)
    _compare(x, b[2].arrays(), tol=1e-8)
    for n in ('sltend', 'qltend'):
        p, q = getattr(a[4], n), getattr(b[4], n)
        assert np.max(np.abs(p - q)) <= 1e-4 * (np.max(np.abs(p)) or 1.0), n
