"""Randomised invariants of the oracle: over random soundings, surface
fluxes, winds, seeds and moisture the column water and energy identities of
check_energy_chng close, every column finishes with status ok and finite
outputs, and the returned state keeps its physical ranges.  These pin the
restatement where no reference outputs exist."""
import numpy as np
import pytest

import oracle
from crm_gb300 import gcm_coupling as G
from crm_gb300 import synthetic as S


def _case(seed):
    rng = np.random.default_rng(1000 + seed)
    cfg = S.config_32x28()
    ncol = 3
    t_sfc = rng.uniform(275.0, 305.0, ncol)
    shf = rng.uniform(0.0, 40.0, ncol)
    lhf = rng.uniform(0.0, 200.0, ncol)
    u_top = float(rng.uniform(-15.0, 15.0))
    moist = bool(rng.integers(2))
    dt_gl = float(rng.choice([400.0, 800.0, 1200.0]))
    cin, st, rad, desc = S.make_inputs(cfg, ncol, t_sfc, shf, lhf, dt_gl=dt_gl, seed=seed,
                                       u_top=u_top, moist=moist)
    return cfg, cin, st, rad, desc, ncol


@pytest.mark.parametrize('seed', range(8))
def test_identities_and_ranges_hold_for_random_columns(seed):
    cfg, cin, st, rad, desc, ncol = _case(seed)
    rad_in = rad.copy()
    rc, stat, out = oracle.run(cfg, desc, cin, st, rad)
    assert rc == 0 and np.all(np.asarray(stat) == 0), stat
    for n, a in out.arrays().items():
        assert np.isfinite(a).all(), n
    for n, a in st.arrays().items():
        assert np.isfinite(a[:ncol]).all(), n
    # water: column tendency + surface precipitation + storage = 0
    rw = G.water_residual(cin, out, ncol) / G.water_scale(cin, out, ncol)
    assert np.max(np.abs(rw)) < 1e-9, rw
    # energy: tendency = radiation + latent heat of precipitation and storage
    re = G.energy_residual(cin, rad_in, out, ncol, cfg.crm_nz) / \
        G.energy_scale(cin, rad_in, out, ncol, cfg.crm_nz)
    assert np.max(np.abs(re)) < 1e-6, re
    # physical ranges of the returned state
    assert np.all(st.qt[:ncol] >= 0.0) and np.all(st.qp[:ncol] >= 0.0)
    assert np.all(st.qn[:ncol] >= 0.0)
    assert 150.0 < st.temperature[:ncol].min() and st.temperature[:ncol].max() < 340.0
    assert np.all(out.precc[:ncol] >= 0.0) and np.all(out.precl[:ncol] >= 0.0)
