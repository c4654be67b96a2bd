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
CRM's column qp over the call, crm_module.F90:1086-1100).  This module states
the tendency, the update and that residual.
"""
import numpy as np

GRAVIT = 9.80616       # shr_const_g
CPAIR = 1.00464e3      # shr_const_cpdair
RHO_WATER = 1000.0     # precipitation rates are m/s of liquid water


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
