"""GCM side of the CRM call: the column water and energy identities of
check_energy_chng hold for the oracle's output (FP64), and a few GCM steps of
tendencies applied between calls keep them."""
import numpy as np

import oracle
from crm_gb300 import gcm_coupling as G
from crm_gb300 import synthetic as S


def test_water_identity_holds():
    for wl in (S.workload_32x28, S.workload_64x58):
        cfg, cin, st, rad, desc = wl(ncrms=3, moist=True)
        rc, stat, out = oracle.run(cfg, desc, cin, st, rad)
        assert rc == 0
        r = G.water_residual(cin, out, 3)
        assert np.all(np.abs(r) <= 1e-9 * G.water_scale(cin, out, 3)), r


def test_coupled_steps_keep_the_identity():
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=2, moist=True)
    for igstep in (1, 2, 3):
        desc.igstep = igstep
        rc, stat, out = oracle.run(cfg, desc, cin, st, rad)
        assert rc == 0
        r = G.water_residual(cin, out, 2)
        assert np.all(np.abs(r) <= 1e-9 * G.water_scale(cin, out, 2)), (igstep, r)
        t0 = cin.tl.copy()
        G.apply_ptend(cin, G.ptend(out, 2), desc.dt_gl)
        assert not np.array_equal(t0, cin.tl)
        assert np.all(cin.ql >= 0)


def test_energy_identity_holds():
    for wl, moist in ((S.workload_32x28, False), (S.workload_32x28, True), (S.workload_64x58, True)):
        cfg, cin, st, rad, desc = wl(ncrms=3, moist=moist)
        rad_in = rad.copy()
        rc, stat, out = oracle.run(cfg, desc, cin, st, rad)
        assert rc == 0
        r = G.energy_residual(cin, rad_in, out, 3, cfg.crm_nz)
        scale = G.energy_scale(cin, rad_in, out, 3, cfg.crm_nz)
        assert np.all(np.abs(r) <= 1e-7 * scale), (wl.__name__, moist, r / scale)


def test_energy_identity_detects_a_missing_term():
    """The identity is not vacuous: dropping the surface precipitation term
    of a precipitating column leaves a residual of its size."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=2, moist=True)
    rad_in = rad.copy()
    rc, stat, out = oracle.run(cfg, desc, cin, st, rad)
    assert rc == 0
    out.precc[:] = 0.0
    out.precl[:] = 0.0
    r = G.energy_residual(cin, rad_in, out, 2, cfg.crm_nz)
    assert np.all(np.abs(r) > 1e-3 * G.energy_scale(cin, rad_in, out, 2, cfg.crm_nz))
