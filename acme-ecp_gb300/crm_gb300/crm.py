"""The reference's crm() entry, restated for a Python host.

    crm(lchnk, icol, ncrms, dt_gl, plev, crm_input, crm_state, crm_rad,
        crm_output, config=..., gcol=..., igstep=...)

mirrors subroutine crm in components/cam/src/physics/crm/crm_module.F90:45-56
(argument meaning and order kept; crm_ecpp_output is absent because ECPP is
off).  The Fortran version reads get_gcol_p, get_nstep and the CPP grid
constants from modules (crm_module.F90:33,286-291,679); here they are the
explicit `gcol`, `igstep` and `config` arguments.  crm_state and crm_rad are
updated in place and crm_output is overwritten, as in the reference.  The
return value is the per-column status array (all CRM_OK on success); the
reference stops the model instead (kurant.F90:66-75).
"""
from . import crm_types as T
from .lib import CrmContext, CrmError

_contexts = {}


def _key(cfg):
    return tuple(sorted(cfg.__dict__.items()))


def get_context(cfg: T.CrmConfig):
    """A cached handle per configuration (the reference builds one binary per
    (nx, ny, nz, dx, dt, microphysics) combination)."""
    k = _key(cfg)
    ctx = _contexts.get(k)
    if ctx is None:
        ctx = CrmContext(cfg)
        _contexts[k] = ctx
    return ctx


def crm(lchnk, icol, ncrms, dt_gl, plev, crm_input, crm_state, crm_rad, crm_output,
        config: T.CrmConfig, gcol=None, igstep=2, raise_on_error=True):
    """Advance ncrms CRMs over one GCM step dt_gl (see module docstring)."""
    if plev != config.plev:
        raise ValueError('plev %d does not match the configuration (%d)' % (plev, config.plev))
    ld = crm_input.ld
    if gcol is None:
        gcol = [int(i) + 1 for i in icol]
    if config.max_ncrms < ld:
        config = T.CrmConfig(**{**config.__dict__, 'max_ncrms': ld})
    ctx = get_context(config)
    desc = T.call_desc(ncrms, ld, dt_gl, igstep, gcol, lchnk=lchnk)
    status = ctx.run(desc, crm_input, crm_state, crm_rad, crm_output)
    if raise_on_error and ctx.last_rc != T.CRM_OK:
        raise CrmError(ctx.last_rc, 'crm')
    return status
