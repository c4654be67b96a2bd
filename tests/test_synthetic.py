"""The synthetic workloads are the soundings they claim to be: the stated
lapse rate and tropopause floor, relative humidity profile, wind shear,
surface-flux forcing of the lowest GCM layer, radiative cooling, the seeded
+-0.1 K perturbation of the lowest four CRM levels, and (64 x 58 batch) the
latitude-dependent surface temperature and fluxes."""
import numpy as np

from crm_gb300 import synthetic as S


def test_sounding_profiles():
    s = S.sounding(30, 300.0, u_top=10.0)
    z = s['zmid']
    assert np.all(np.diff(z) < 0)                      # top to bottom
    expect_t = np.maximum(300.0 - 6.5e-3 * z, 200.0)
    assert np.allclose(s['t'], expect_t, rtol=0, atol=1e-9)
    rh = s['q'] / S.qsatw(s['t'], s['pmid'] / 100.0)
    expect_rh = np.where(z < 12000.0, 0.8 - 0.7 * z / 12000.0, 0.1)
    assert np.allclose(rh, expect_rh, rtol=1e-12)
    assert np.allclose(s['u'], 10.0 * np.minimum(z, 12000.0) / 12000.0)
    assert np.all(s['v'] == 0.0)
    # hydrostatic heights: the interfaces bracket the midpoints
    assert np.all(s['zint'][1:] < z) and np.all(z < s['zint'][:-1])
    assert s['zint'][-1] == 0.0


def test_inputs_forcing_and_perturbation():
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=3)
    s = S.sounding(cfg.plev, 300.0)
    # surface fluxes heat and moisten the lowest GCM layer over one GCM step
    g_dp = S.GRAV / s['pdel'][-1]
    assert np.isclose(cin.tl[0, -1] - s['t'][-1], g_dp * 10.0 / S.CPAIR * desc.dt_gl)
    assert np.isclose(cin.ql[0, -1] - s['q'][-1], g_dp * 100.0 / S.LATVAP * desc.dt_gl)
    assert np.allclose(cin.tl[0, :-1], s['t'][:-1])
    # CRM state: the sounding on CRM levels, lowest four levels perturbed
    k_gcm = cfg.plev - 1 - np.arange(cfg.crm_nz)        # CRM level k -> GCM index
    base = s['t'][k_gcm]
    d = st.temperature[:3, :, 0, :] - base[None, None, :]
    assert np.all(np.abs(d[:, :, :4]) <= 0.1) and np.any(np.abs(d[:, :, :4]) > 0.05)
    assert np.all(d[:, :, 4:] == 0.0)
    assert not np.array_equal(d[0], d[1])               # seeded per column
    # radiative cooling below 12 km, none above
    qr = rad.qrad[0, 0, 0, :]
    z = s['zmid'][k_gcm]
    assert np.allclose(qr[z < 12000.0], -1.5 / 86400.0) and np.all(qr[z >= 12000.0] == 0.0)


def test_batch_64x58_latitudes():
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=64)
    assert (cfg.crm_nx, cfg.crm_nz, cfg.plev, cfg.crm_dx, cfg.crm_dt) == (64, 58, 72, 1000.0, 10.0)
    # lowest-level CRM temperature (before the perturbation) spans the
    # 271 + 29 cos(lat) range of lat in [-60, 60] degrees
    t_bot = np.median(st.temperature[:64, :, 0, 0], axis=1)
    z_bot = np.array([S.sounding(72, 300.0)['zmid'][-1]])
    t_sfc = t_bot + 6.5e-3 * z_bot
    assert t_sfc.min() > 271.0 + 29.0 * 0.5 - 0.2 and t_sfc.max() < 300.0 + 0.2
    assert t_sfc.max() - t_sfc.min() > 5.0
