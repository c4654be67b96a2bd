"""Build and call the CPU FP64 restatement of crm() (crm_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the library itself.

PARITY UNPINNED: no reference outputs exist to check the restatement against
(no golden vectors in the reference, no Fortran compiler to run it); it is
held to conservation identities and mathematical properties instead.

The restatement is compiled with -ffp-contract=off so that every floating
point operation is a separately rounded IEEE operation, the same contract the
FP64 device form is compiled with (nvcc -fmad=false).
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB = os.path.join(HERE, 'liboracle_crm.so')
SRC = [os.path.join(HERE, 'crm_oracle.cpp'), os.path.join(HERE, 'oracle_core.h'),
       os.path.join(REPO, 'include', 'crm_gb300.h'), os.path.join(REPO, 'include', 'crm_detmath.h')]

sys.path.insert(0, os.path.join(REPO, 'acme-ecp_gb300'))
from crm_gb300 import crm_types as T  # noqa: E402

_lib = None


def build(force=False, check=False):
    """Compile liboracle_crm.so (a few seconds).  check=True adds array
    bounds checks (slower) into a separate library."""
    out = LIB if not check else LIB.replace('.so', '_chk.so')
    if not force and os.path.exists(out) and all(
            os.path.getmtime(out) >= os.path.getmtime(s) for s in SRC):
        return out
    cmd = ['g++', '-O2', '-std=c++17', '-ffp-contract=off', '-fno-fast-math',
           '-fopenmp', '-fPIC', '-shared', '-o', out, SRC[0]]
    if check:
        cmd.insert(1, '-DORACLE_CHECK')
    subprocess.check_call(cmd)
    return out


def load(check=False):
    global _lib
    if _lib is None or check:
        lib = C.CDLL(build(check=check))
        lib.oracle_crm_run.restype = C.c_int
        lib.oracle_crm_run.argtypes = [C.POINTER(T.CCrmConfig), C.POINTER(T.CCrmCallDesc),
                                       C.POINTER(T.CCrmInput), C.POINTER(T.CCrmState),
                                       C.POINTER(T.CCrmRad), C.POINTER(T.CCrmOutput),
                                       C.POINTER(C.c_int), C.c_int]
        lib.oracle_rng_mt.restype = C.c_int
        lib.oracle_rng_mt.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double)]
        lib.oracle_sat.restype = C.c_int
        lib.oracle_sat.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int,
                                   C.POINTER(C.c_double)]
        lib.oracle_gammafff.restype = C.c_float
        lib.oracle_gammafff.argtypes = [C.c_float]
        lib.oracle_fft991.restype = C.c_int
        lib.oracle_fft991.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_int]
        if check:
            return lib
        _lib = lib
    return _lib


def run(cfg, desc, cin, state, rad, out=None, nthreads=0, check=False):
    """Run the oracle in place on state/rad; returns (rc, col_status, out)."""
    lib = load(check=check)
    ncrms = desc.ncrms
    if out is None:
        out = T.CrmOutput(desc.ld, cfg.crm_nx, cfg.crm_ny, cfg.crm_nz, cfg.plev)
    status = np.zeros(ncrms, dtype=np.int32)
    c_cfg = cfg.to_c()
    c_in, c_st, c_rad, c_out = cin.to_c(), state.to_c(), rad.to_c(), out.to_c()
    rc = lib.oracle_crm_run(C.byref(c_cfg), C.byref(desc), C.byref(c_in), C.byref(c_st),
                            C.byref(c_rad), C.byref(c_out),
                            status.ctypes.data_as(C.POINTER(C.c_int)), int(nthreads))
    return rc, status, out


def fft991(x, isign):
    """The oracle's fft991 on one vector (len n + 2, float64, modified in
    place copy): isign -1 grid point -> spectral, +1 back."""
    import numpy as np
    a = np.ascontiguousarray(np.array(x, dtype=np.float64))
    rc = load().oracle_fft991(a.ctypes.data_as(C.POINTER(C.c_double)), a.size - 2, int(isign))
    if rc != 0:
        raise ValueError('fft991: unsupported length %d' % (a.size - 2))
    return a


def rng_mt(seed, n):
    """n draws of the oracle's RNG_MT after set_seed(seed)."""
    out = np.zeros(n)
    rc = load().oracle_rng_mt(int(seed), int(n), out.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0
    return out


SAT_FUNCS = ('esatw', 'esati', 'dtesatw', 'dtesati', 'qsatw', 'qsati', 'dtqsatw', 'dtqsati')


def sat(name, t, p=None):
    """The oracle's sat.F90 function `name` at temperatures t (pressures p)."""
    t = np.ascontiguousarray(t, dtype=np.float64)
    pp = None if p is None else np.ascontiguousarray(p, dtype=np.float64)
    out = np.zeros_like(t)
    rc = load().oracle_sat(SAT_FUNCS.index(name), t.ctypes.data_as(C.POINTER(C.c_double)),
                           None if pp is None else pp.ctypes.data_as(C.POINTER(C.c_double)),
                           t.size, out.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0
    return out


def gammafff(x):
    """The oracle's gammafff (crm/gammafff.c) for float arguments."""
    lib = load()
    return np.array([lib.oracle_gammafff(float(v)) for v in np.atleast_1d(x)], dtype=np.float32)

