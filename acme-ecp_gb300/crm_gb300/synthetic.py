"""Seeded synthetic GCM columns for the CRM workloads.

The reference measures on no dataset; its production shapes are the SP
compsets in components/cam/cime_config/config_component.xml:100-117
(FSP*FAST: 30 GCM levels, crm_nz 28, dx 4 km, dt 20 s; FSP*V1: 72 levels,
crm_nz 58, dx 1 km).  These helpers build the inputs crm() receives from
crm_physics_tend (components/cam/src/physics/cam/crm_physics.F90:1051-1130)
for an idealised sounding:

  * hybrid levels from the E3SM tables (data/vcoord.json), P0 = ps = 1000 hPa;
  * T = max(T_sfc - 6.5 K/km z, 200 K); RH 80 % at the surface falling
    linearly to 10 % at 12 km and 10 % above; q = RH * qsat_w(T, p);
  * u rising linearly 0 -> u_top over 0-12 km, constant above (v likewise
    with v_top); heights from hydrostatic balance of the virtual temperature;
  * surface fluxes SHF/LHF applied to the lowest GCM layer over one GCM step,
    as crm_surface_flux_bypass_tend does (crm_physics.F90:1653-1704), and
    bflxls = SHF/cp + 0.61 T_bot LHF/L_v, tau00 = 0, wndls = |u_bot|;
  * the CRM state starts horizontally uniform from the sounding
    (crm_physics.F90:912-939) plus a seeded uniform +-0.1 K perturbation of
    the lowest 4 CRM levels; crm_rad%qrad = -1.5 K/day below 12 km.
"""
import json
import os

import numpy as np

from .crm_types import CrmConfig, CrmInput, CrmRad, CrmState, call_desc

CPAIR = 1.00464e3
GRAV = 9.80616
LATVAP = 2.501e6
RDAIR = 6.02214e26 * 1.38065e-23 / 28.966
RH2O = 6.02214e26 * 1.38065e-23 / 18.016
ZVIR = RH2O / RDAIR - 1.0

_VC = None


def vcoord(nlev):
    global _VC
    if _VC is None:
        with open(os.path.join(os.path.dirname(__file__), 'data', 'vcoord.json')) as f:
            _VC = json.load(f)
    d = _VC['L%d' % nlev]
    return {k: np.asarray(v) if isinstance(v, list) else v for k, v in d.items()}


def qsatw(t, p_mb):
    """Flatau et al. (1992) saturation mixing ratio over water."""
    a = [6.105851, 0.4440316, 0.1430341e-1, 0.2641412e-3, 0.2995057e-5,
         0.2031998e-7, 0.6936113e-10, 0.2564861e-13, -0.3704404e-15]
    dt = np.maximum(t - 273.16, -80.0)
    es = a[8]
    for c in reversed(a[:8]):
        es = c + dt * es
    return 0.622 * es / np.maximum(es, p_mb - es)


def sounding(plev, t_sfc, u_top=10.0, v_top=0.0, ps=1.0e5):
    """One GCM column, top-to-bottom (index 0 = model top, as in CAM)."""
    vc = vcoord(plev)
    p0 = vc['p0']
    pint = vc['hyai'] * p0 + vc['hybi'] * ps
    pmid = vc['hyam'] * p0 + vc['hybm'] * ps
    pdel = np.diff(pint)
    t = np.full(plev, t_sfc)
    q = np.zeros(plev)
    zint = np.zeros(plev + 1)
    zmid = np.zeros(plev)
    for _ in range(8):                       # fixed point of T(z(T))
        tv = t * (1.0 + ZVIR * q)
        zint[plev] = 0.0
        for k in range(plev - 1, -1, -1):
            zint[k] = zint[k + 1] + RDAIR * tv[k] / GRAV * np.log(pint[k + 1] / pint[k])
            zmid[k] = zint[k + 1] + RDAIR * tv[k] / GRAV * np.log(pint[k + 1] / pmid[k])
        t = np.maximum(t_sfc - 6.5e-3 * zmid, 200.0)
        rh = np.where(zmid < 12000.0, 0.8 - 0.7 * zmid / 12000.0, 0.1)
        q = rh * qsatw(t, pmid / 100.0)
    frac = np.minimum(zmid, 12000.0) / 12000.0
    return dict(pint=pint, pmid=pmid, pdel=pdel, t=t, q=q, zint=zint,
                zmid=zmid, u=u_top * frac, v=v_top * frac, ps=ps)


def make_inputs(cfg: CrmConfig, ncrms, t_sfc, shf, lhf, dt_gl=1200.0, seed=0,
                u_top=10.0, v_top=0.0, ld=None, gcol0=1, moist=False):
    """Build (crm_input, crm_state, crm_rad, desc) for ncrms columns.

    t_sfc, shf, lhf: scalars or arrays of length ncrms.  Column c uses
    numpy PCG64(seed + c) for its +-0.1 K state perturbation and the
    reference's own setperturb (seed gcol*1000, gcol = gcol0 + c) runs
    inside crm() because igstep = 1.

    moist=True makes a test state that exercises every microphysics branch
    from the first step: total water 3 % above saturation between 1 and
    4 km and between 7 and 9 km (liquid and ice cloud), precipitation
    1e-3 kg/kg between 2 and 5 km, and GCM cloud water/ice inputs.
    """
    ld = ld or ncrms
    plev, nx, ny, nz = cfg.plev, cfg.crm_nx, cfg.crm_ny, cfg.crm_nz
    t_sfc = np.broadcast_to(np.asarray(t_sfc, float), (ncrms,))
    shf = np.broadcast_to(np.asarray(shf, float), (ncrms,))
    lhf = np.broadcast_to(np.asarray(lhf, float), (ncrms,))
    cin = CrmInput.zeros(ld, plev)
    st = CrmState.zeros(ld, nx, ny, nz)
    rad = CrmRad.zeros(ld, cfg.crm_nx_rad, cfg.crm_ny_rad, nz)
    for c in range(ncrms):
        s = sounding(plev, float(t_sfc[c]), u_top, v_top)
        # CRM state from the sounding before the surface-flux update
        for k in range(nz):
            m = plev - 1 - k
            st.u_wind[c, :, :, k] = s['u'][m]
            st.v_wind[c, :, :, k] = s['v'][m]
            st.temperature[c, :, :, k] = s['t'][m]
            st.qt[c, :, :, k] = s['q'][m]
            rad.qrad[c, :, :, k] = -1.5 / 86400.0 if s['zmid'][m] < 12000.0 else 0.0
        rng = np.random.Generator(np.random.PCG64(seed + c))
        st.temperature[c, :, :, :4] += rng.uniform(-0.1, 0.1, size=(nx, ny, 4))
        if moist:
            for k in range(nz):
                m = plev - 1 - k
                z = s['zmid'][m]
                qs = qsatw(s['t'][m], s['pmid'][m] / 100.0)
                if 1000.0 < z < 4000.0 or 7000.0 < z < 9000.0:
                    st.qt[c, :, :, k] = 1.03 * qs * (1.0 + 0.02 * rng.uniform(-1, 1, size=(nx, ny)))
                if 2000.0 < z < 5000.0:
                    st.qp[c, :, :, k] = 1.0e-3 * rng.uniform(0.5, 1.0, size=(nx, ny))
        # surface fluxes applied to the lowest GCM layer over one GCM step
        t = s['t'].copy()
        q = s['q'].copy()
        g_dp = GRAV / s['pdel'][-1]
        t[-1] += g_dp * shf[c] / CPAIR * dt_gl
        q[-1] += g_dp * lhf[c] / LATVAP * dt_gl
        cin.zmid[c] = s['zmid']
        cin.zint[c] = s['zint']
        cin.tl[c] = t
        cin.ql[c] = q
        if moist:
            cin.qccl[c] = np.where((s['zmid'] > 1000.0) & (s['zmid'] < 4000.0), 2.0e-5, 0.0)
            cin.qiil[c] = np.where((s['zmid'] > 7000.0) & (s['zmid'] < 9000.0), 1.0e-5, 0.0)
        cin.ps[c] = s['ps']
        cin.pmid[c] = s['pmid']
        cin.pint[c] = s['pint']
        cin.pdel[c] = s['pdel']
        cin.ul[c] = s['u']
        cin.vl[c] = s['v']
        cin.ocnfrac[c] = 1.0
        cin.bflxls[c] = shf[c] / CPAIR + 0.61 * t[-1] * lhf[c] / LATVAP
        cin.wndls[c] = np.hypot(s['u'][-1], s['v'][-1])
        cin.fluxt00[c] = shf[c] / CPAIR
        cin.fluxq00[c] = lhf[c] / LATVAP
    desc = call_desc(ncrms, ld, dt_gl, igstep=1, gcol=np.arange(gcol0, gcol0 + ncrms))
    return cin, st, rad, desc


def config_32x28(precision=0, batch_mode=0):
    """Plain 2D CRM, FAST-compset shape: nx 32, nz 28 of 30 levels, dx 4 km, dt 20 s."""
    return CrmConfig(crm_nx=32, crm_ny=1, crm_nz=28, plev=30, crm_dx=4000.0,
                     crm_dt=20.0, precision=precision, batch_mode=batch_mode)


def config_64x58(precision=0, batch_mode=0, nx=64):
    """2D CRM, V1-compset shape: nx 64, nz 58 of 72 levels, dx 1 km, dt 10 s."""
    return CrmConfig(crm_nx=nx, crm_ny=1, crm_nz=58, plev=72, crm_dx=1000.0,
                     crm_dt=10.0, precision=precision, batch_mode=batch_mode)


def workload_32x28(ncrms=16, seed=0, moist=False, **kw):
    """16 columns, T_sfc 300 K, SHF 10 W/m2, LHF 100 W/m2."""
    cfg = config_32x28(**kw)
    return (cfg,) + make_inputs(cfg, ncrms, 300.0, 10.0, 100.0, seed=seed, moist=moist)


def workload_64x58(ncrms=1024, seed=0, nx=64, moist=False, gcol0=1, **kw):
    """lat ~ U[-60, 60] deg (seeded), T_sfc = 271 + 29 cos(lat), fluxes * cos(lat)."""
    cfg = config_64x58(nx=nx, **kw)
    rng = np.random.Generator(np.random.PCG64(10_000 + seed))
    lat = rng.uniform(-60.0, 60.0, size=ncrms)
    cl = np.cos(np.deg2rad(lat))
    return (cfg,) + make_inputs(cfg, ncrms, 271.0 + 29.0 * cl, 10.0 * cl,
                                100.0 * cl, seed=seed, moist=moist, gcol0=gcol0)


def config_3d(precision=0, batch_mode=0, nx=32, ny=32, nz=58, dx=2000.0):
    """3D CRM: nx x ny x nz of 72 levels, dx = dy = 2 km, dt 10 s."""
    return CrmConfig(crm_nx=nx, crm_ny=ny, crm_nz=nz, plev=72, crm_dx=dx, crm_dy=dx,
                     crm_dt=10.0, precision=precision, batch_mode=batch_mode)


def workload_3d(ncrms=256, seed=0, nx=32, ny=32, nz=58, moist=False, gcol0=1, **kw):
    """The 64 x 58 workload's soundings (lat ~ U[-60, 60] deg, T_sfc = 271 +
    29 cos(lat), fluxes * cos(lat)) with v rising 0 -> 5 m/s over 0-12 km."""
    cfg = config_3d(nx=nx, ny=ny, nz=nz, **kw)
    rng = np.random.Generator(np.random.PCG64(10_000 + seed))
    lat = rng.uniform(-60.0, 60.0, size=ncrms)
    cl = np.cos(np.deg2rad(lat))
    return (cfg,) + make_inputs(cfg, ncrms, 271.0 + 29.0 * cl, 10.0 * cl,
                                100.0 * cl, seed=seed, moist=moist, gcol0=gcol0, v_top=5.0)
