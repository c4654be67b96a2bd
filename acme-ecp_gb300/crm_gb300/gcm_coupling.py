"""The GCM side of a CRM call: physics tendencies and the budget check.

After crm() returns, crm_physics_tend (components/cam/src/physics/cam/
crm_physics.F90:1163-1300) turns the CRM output into a physics tendency —
ptend%s = sltend, ptend%q(:,:,1) = qltend, q(ixcldliq) = qcltend,
q(ixcldice) = qiltend — that physics_update applies over the GCM step, and
check_energy_chng (components/cam/src/physics/cam/check_energy.F90:358-561)
verifies that the column's water changed only by the surface fluxes.  For
the CRM the water identity is exact:

    sum_k pdel_k / g (qltend + qcltend + qiltend)_k
        = - (precc + precl) * rho_water - prectend

i.e. the GCM column loses what fell out at the surface plus what is still
stored in the CRM as precipitating water (prectend is the change of the
CRM's column qp over the call, crm_module.F90:1086-1100).

The energy side of check_energy_chng closes the same way.  Inside the CRM
the liquid-ice static energy t (crm_module.F90:508-509) changes only by the
large-scale forcing (which returns the column to the GCM state), the
radiative heating qrad (crm_module.F90:766-777) and the latent heat carried
out by precipitation at the surface (precip_fall, ice_fall); damping keeps
the level means, advection and SGS diffusion conserve it, and condensation
and precipitation processes leave it unchanged.  Writing tabs from t at the
end of the call gives, per column [W/m2],

    sum_k pdel_k / g (sltend - Lc qcltend - Ls qiltend)
        = cp sum_k pdel_k / g <qrad>_k
          + rho_water (Lc (precc + precl) + Lf (precsc + precsl))
          + Lc prectend + Lf precstend

with the CRM's own latent heats (crm/params.F90:49-55) and the levels
whose tendencies crm() zeroes (the top two) left out of the qrad sum.
This module states the tendency, the update and both residuals.
"""
import numpy as np

GRAVIT = 9.80616       # shr_const_g
CPAIR = 1.00464e3      # shr_const_cpdair
RHO_WATER = 1000.0     # precipitation rates are m/s of liquid water
LCOND = 2.501e6        # CRM latent heats (crm/params.F90, CRM branch)
LFUS = 3.337e5
LSUB = LCOND + LFUS


def ptend(out, ncol):
    """The physics tendency of the CRM call for the first ncol columns:
    {'s': dry static energy [W/kg], 'q', 'qc', 'qi': [kg/kg/s]} on the GCM
    levels (the CRM sets the two levels above its top to zero)."""
    return {'s': np.array(out.sltend[:ncol]), 'q': np.array(out.qltend[:ncol]),
            'qc': np.array(out.qcltend[:ncol]), 'qi': np.array(out.qiltend[:ncol])}


def apply_ptend(cin, pt, dt_gl):
    """physics_update on the crm_input profiles (the GCM state the next call
    sees): T += s/cp dt, q += q dt, clipping the water species at zero."""
    n = pt['s'].shape[0]
    cin.tl[:n] += pt['s'] / CPAIR * dt_gl
    cin.ql[:n] = np.maximum(cin.ql[:n] + pt['q'] * dt_gl, 0.0)
    cin.qccl[:n] = np.maximum(cin.qccl[:n] + pt['qc'] * dt_gl, 0.0)
    cin.qiil[:n] = np.maximum(cin.qiil[:n] + pt['qi'] * dt_gl, 0.0)
    return cin


def water_residual(cin, out, ncol):
    """Per column [kg/m2/s]: column water tendency + surface precipitation
    + CRM precipitation storage tendency (zero up to rounding)."""
    pd = np.asarray(cin.pdel[:ncol]) / GRAVIT
    dw = np.sum(pd * (out.qltend[:ncol] + out.qcltend[:ncol] + out.qiltend[:ncol]), axis=1)
    prec = (out.precc[:ncol] + out.precl[:ncol]) * RHO_WATER
    return dw + prec + out.prectend[:ncol]


def water_scale(cin, out, ncol):
    """Magnitude of the terms of water_residual, to make it relative."""
    pd = np.asarray(cin.pdel[:ncol]) / GRAVIT
    dw = np.sum(pd * np.abs(out.qltend[:ncol] + out.qcltend[:ncol] + out.qiltend[:ncol]), axis=1)
    return dw + np.abs((out.precc[:ncol] + out.precl[:ncol]) * RHO_WATER) + np.abs(out.prectend[:ncol])


def _energy_terms(cin, rad, out, ncol, nzm):
    pd = np.asarray(cin.pdel[:ncol]) / GRAVIT
    plev = pd.shape[1]
    lhs = np.sum(pd * (out.sltend[:ncol] - LCOND * out.qcltend[:ncol] - LSUB * out.qiltend[:ncol]), axis=1)
    qr = np.asarray(rad.qrad[:ncol, :, 0, :]).mean(axis=1)       # (ncol, crm_nz), K/s
    rad_heat = np.zeros(ncol)
    for k in range(1, nzm - 1):              # CRM level k is GCM level plev - k + 1
        rad_heat += pd[:, plev - k] * CPAIR * qr[:, k - 1]
    prec = RHO_WATER * (LCOND * (out.precc[:ncol] + out.precl[:ncol]) +
                        LFUS * (out.precsc[:ncol] + out.precsl[:ncol]))
    store = LCOND * out.prectend[:ncol] + LFUS * out.precstend[:ncol]
    return lhs, rad_heat, prec, store


def energy_residual(cin, rad, out, ncol, nzm):
    """Per column [W/m2]: column energy tendency - radiative heating - latent
    heat of the surface precipitation - latent heat of the CRM's precipitation
    storage change (zero up to rounding).  rad holds the qrad the call was
    given; nzm = crm_nz."""
    lhs, rad_heat, prec, store = _energy_terms(cin, rad, out, ncol, nzm)
    return lhs - rad_heat - prec - store


def energy_scale(cin, rad, out, ncol, nzm):
    """Magnitude of the terms of energy_residual, to make it relative."""
    pd = np.asarray(cin.pdel[:ncol]) / GRAVIT
    _, rad_heat, prec, store = _energy_terms(cin, rad, out, ncol, nzm)
    dw = np.sum(pd * np.abs(out.sltend[:ncol]), axis=1)
    return dw + np.abs(rad_heat) + np.abs(prec) + np.abs(store)
