"""Host-side mirror of the reference's CRM derived types and of the C ABI.

The reference passes four Fortran derived types to crm():
  crm_input_type   components/cam/src/physics/crm/crm_input_module.F90:10-47
  crm_state_type   components/cam/src/physics/crm/crm_state_module.F90:12-56
  crm_rad_type     components/cam/src/physics/crm/crm_rad_module.F90:17-34
  crm_output_type  components/cam/src/physics/crm/crm_output_module.F90:7-133
Each class below holds the same components as numpy arrays in Fortran order
(column index fastest), so the buffers can be handed to the C ABI
(include/crm_gb300.h) without copies.
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

# enum crm_status
CRM_OK = 0
CRM_ERR_ARG = 1
CRM_ERR_CFL = 2
CRM_ERR_NONFINITE = 3
CRM_ERR_CUDA = 4
CRM_ERR_UNSUPPORTED = 5
CRM_ERR_TIMEOUT = 6
CRM_ERR_BUDGET = 7
CRM_ERR_NO_DEVICE = 8
CRM_ERR_TOO_LARGE = 9
CRM_PENDING = 10

CRM_MICRO_SAM1MOM = 0
CRM_MICRO_M2005 = 1
CRM_FP64 = 0
CRM_FP32_MIXED = 1
CRM_FP64_FMA = 2
CRM_PER_COLUMN = 0
CRM_REFERENCE_BATCH = 1

# enum crm_output_field, in order, with the shape class of each field
OUTPUT_FIELDS = (
    [(n, '4d') for n in ('qcl', 'qci', 'qpl', 'qpi', 'tk', 'tkh')] +
    [('prec_crm', '3d')] +
    [(n, '1d') for n in ('cltot', 'clhgh', 'clmed', 'cllow', 'precc', 'precl',
                         'precsc', 'precsl', 'jt_crm', 'mx_crm', 'prectend',
                         'precstend', 'taux', 'tauy', 'z0m', 'timing_factor')] +
    [(n, '2d') for n in ('cldtop', 'qc_mean', 'qi_mean', 'qs_mean', 'qg_mean',
                         'qr_mean', 'sltend', 'qltend', 'qcltend', 'qiltend',
                         'cld', 'gicewp', 'gliqwp', 'mctot', 'mcup', 'mcdn',
                         'mcuup', 'mcudn', 'mu_crm', 'md_crm', 'du_crm',
                         'eu_crm', 'ed_crm', 'flux_qt', 'fluxsgs_qt', 'tkez',
                         'tkesgsz', 'tkz', 'flux_u', 'flux_v', 'flux_qp',
                         'precflux', 'qt_ls', 'qt_trans', 'qp_trans',
                         'qp_fall', 'qp_src', 'qp_evp', 't_ls')])
CRM_NOUT = len(OUTPUT_FIELDS)

# phases timed by a profiling build (enum PhaseId in csrc/crm_kernel.h)
PHASE_NAMES = ('init', 'kurant', 'buoyancy', 'forcing', 'damping', 'ice_fall', 'bound',
               'tke', 'adv_mom', 'diff_mom', 'press_rhs', 'fft_fwd', 'tridiag', 'fft_inv',
               'press_grad', 'adams', 'adv_t', 'adv_qt', 'adv_qp', 'fall1', 'fall2', 'uvw',
               'diff_t', 'diff_q', 'prec_init', 'cloud', 'prec_proc', 'micro_diag', 'diagnose',
               'stats', 'final')

INPUT_FIELDS = ('zmid', 'zint', 'tl', 'ql', 'qccl', 'qiil', 'ps', 'pmid',
                'pint', 'pdel', 'phis', 'ul', 'vl', 'ocnfrac', 'tau00',
                'wndls', 'bflxls', 'fluxu00', 'fluxv00', 'fluxt00', 'fluxq00')
STATE_FIELDS = ('u_wind', 'v_wind', 'w_wind', 'temperature', 'qt', 'qp', 'qn')
RAD_FIELDS = ('qrad', 'temperature', 'qv', 'qc', 'qi', 'cld')

_DP = C.POINTER(C.c_double)


class CCrmConfig(C.Structure):
    _fields_ = [('crm_nx', C.c_int), ('crm_ny', C.c_int), ('crm_nz', C.c_int),
                ('crm_nx_rad', C.c_int), ('crm_ny_rad', C.c_int),
                ('plev', C.c_int), ('crm_dx', C.c_double),
                ('crm_dy', C.c_double), ('crm_dt', C.c_double),
                ('microphysics', C.c_int), ('precision', C.c_int),
                ('batch_mode', C.c_int), ('max_ncrms', C.c_int),
                ('use_crm_accel', C.c_int), ('crm_accel_factor', C.c_double),
                ('crm_accel_uv', C.c_int)]


class CCrmInput(C.Structure):
    _fields_ = [(n, _DP) for n in INPUT_FIELDS]


class CCrmState(C.Structure):
    _fields_ = [(n, _DP) for n in STATE_FIELDS]


class CCrmRad(C.Structure):
    _fields_ = [(n, _DP) for n in RAD_FIELDS]


class CCrmOutput(C.Structure):
    _fields_ = [('field', _DP * CRM_NOUT)]


class CCrmCallDesc(C.Structure):
    _fields_ = [('lchnk', C.c_int), ('ncrms', C.c_int), ('ld', C.c_int),
                ('dt_gl', C.c_double), ('igstep', C.c_int),
                ('gcol', C.POINTER(C.c_int)), ('col_map', C.POINTER(C.c_int))]


def _ptr(a):
    assert a.dtype == np.float64 and a.flags.f_contiguous, a.flags
    return a.ctypes.data_as(_DP)


@dataclass
class CrmConfig:
    """Run-time replacement of the reference's CPP build constants
    (bld/configure:1883-1914, crmdims.F90, domain.F90)."""
    crm_nx: int
    crm_ny: int
    crm_nz: int
    plev: int
    crm_dx: float
    crm_dt: float
    crm_dy: float = 0.0
    crm_nx_rad: int = 0
    crm_ny_rad: int = 0
    microphysics: int = CRM_MICRO_SAM1MOM
    precision: int = CRM_FP64
    batch_mode: int = CRM_PER_COLUMN
    max_ncrms: int = 0
    use_crm_accel: int = 0
    crm_accel_factor: float = 0.0
    crm_accel_uv: int = 0

    def __post_init__(self):
        if not self.crm_dy:
            self.crm_dy = self.crm_dx
        if not self.crm_nx_rad:
            self.crm_nx_rad = self.crm_nx
        if not self.crm_ny_rad:
            self.crm_ny_rad = self.crm_ny

    def to_c(self):
        return CCrmConfig(self.crm_nx, self.crm_ny, self.crm_nz,
                          self.crm_nx_rad, self.crm_ny_rad, self.plev,
                          float(self.crm_dx), float(self.crm_dy),
                          float(self.crm_dt), self.microphysics,
                          self.precision, self.batch_mode, self.max_ncrms,
                          int(self.use_crm_accel), float(self.crm_accel_factor),
                          int(self.crm_accel_uv))


class _Bundle:
    """A set of Fortran-ordered float64 arrays with a common leading dim."""
    FIELDS = ()

    def __init__(self, **arrays):
        for n in self.FIELDS:
            setattr(self, n, arrays[n])

    def arrays(self):
        return {n: getattr(self, n) for n in self.FIELDS}

    def copy(self):
        return type(self)(**{n: a.copy(order='F') for n, a in self.arrays().items()})

    def take(self, cols):
        """A new bundle holding the given columns (leading index) in order."""
        cols = np.asarray(cols, dtype=np.int64)
        return type(self)(**{n: np.asfortranarray(a[cols]) for n, a in self.arrays().items()})

    def put(self, cols, other):
        """Write the columns of `other` into columns `cols` of this bundle."""
        cols = np.asarray(cols, dtype=np.int64)
        for n, a in self.arrays().items():
            a[cols] = getattr(other, n)[:len(cols)]

    @property
    def ld(self):
        return getattr(self, self.FIELDS[0]).shape[0]


class CrmInput(_Bundle):
    """crm_input_type: (ld, plev) profiles, zint/pint (ld, plev+1), scalars (ld)."""
    FIELDS = INPUT_FIELDS

    @classmethod
    def zeros(cls, ld, plev):
        a = {}
        for n in INPUT_FIELDS:
            if n in ('zint', 'pint'):
                a[n] = np.zeros((ld, plev + 1), order='F')
            elif n in ('ps', 'phis', 'ocnfrac', 'tau00', 'wndls', 'bflxls',
                       'fluxu00', 'fluxv00', 'fluxt00', 'fluxq00'):
                a[n] = np.zeros((ld,), order='F')
            else:
                a[n] = np.zeros((ld, plev), order='F')
        return cls(**a)

    def to_c(self):
        return CCrmInput(*[_ptr(getattr(self, n)) for n in INPUT_FIELDS])


class CrmState(_Bundle):
    """crm_state_type: (ld, crm_nx, crm_ny, crm_nz) sam1mom prognostics."""
    FIELDS = STATE_FIELDS

    @classmethod
    def zeros(cls, ld, nx, ny, nz):
        return cls(**{n: np.zeros((ld, nx, ny, nz), order='F') for n in STATE_FIELDS})

    def to_c(self):
        return CCrmState(*[_ptr(getattr(self, n)) for n in STATE_FIELDS])


class CrmRad(_Bundle):
    """crm_rad_type: (ld, crm_nx_rad, crm_ny_rad, crm_nz)."""
    FIELDS = RAD_FIELDS

    @classmethod
    def zeros(cls, ld, nx_rad, ny_rad, nz):
        return cls(**{n: np.zeros((ld, nx_rad, ny_rad, nz), order='F') for n in RAD_FIELDS})

    def to_c(self):
        return CCrmRad(*[_ptr(getattr(self, n)) for n in RAD_FIELDS])


class CrmOutput:
    """crm_output_type, sam1mom subset (field order = enum crm_output_field)."""

    def __init__(self, ld, nx, ny, nz, plev):
        self.shape = dict(ld=ld, nx=nx, ny=ny, nz=nz, plev=plev)
        shapes = {'4d': (ld, nx, ny, nz), '3d': (ld, nx, ny), '1d': (ld,),
                  '2d': (ld, plev)}
        for n, s in OUTPUT_FIELDS:
            setattr(self, n, np.zeros(shapes[s], order='F'))

    def arrays(self):
        return {n: getattr(self, n) for n, _ in OUTPUT_FIELDS}

    def to_c(self):
        o = CCrmOutput()
        for i, (n, _) in enumerate(OUTPUT_FIELDS):
            o.field[i] = _ptr(getattr(self, n))
        return o


def call_desc(ncrms, ld, dt_gl, igstep, gcol, lchnk=0):
    """Build the crm_call_desc; keeps the gcol array alive on the result."""
    g = np.ascontiguousarray(gcol, dtype=np.int32)
    d = CCrmCallDesc(lchnk, ncrms, ld, float(dt_gl), igstep,
                     g.ctypes.data_as(C.POINTER(C.c_int)))
    d._keep = g
    return d
