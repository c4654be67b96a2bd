"""Build libcrm_gb300.so (sm_103a) in-tree with nvcc.

Objects, compiled in parallel:
  crm_columns.cu  the column kernel, once per (precision, nx, launch shape)
                  and for the 3D CRM once per (precision, launch shape):
                  FP64 with -fmad=false (bit-identical to a CPU run of the
                  same algorithm), and the FP32-mixed form
  crm_prep.cu     per-column set-up kernel (z0, setperturb draws), -fmad=false
  crm_host.cu     the C ABI (include/crm_gb300.h), host code built with
                  -ffp-contract=off for the same reason
  crm_serve.cu    the continuous-batching service of the C ABI (crm_submit,
                  crm_poll) over resident column slots
  crm_tc_probe.cu crm_debug_tc_transform: the tensor-core transforms of the
                  3D pressure solve on their own
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
CSRC = os.path.join(PKG, 'csrc')
REPO = os.path.dirname(PKG)
LIB = os.path.join(HERE, 'libcrm_gb300.so')
LIB_PROF = os.path.join(HERE, 'libcrm_gb300_prof.so')
OBJ = os.path.join(PKG, '_build')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
COMMON = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC,-ffp-contract=off',
          '-I' + os.path.join(REPO, 'include')]
NUM_SHAPES = 6             # crm_kernel.h kShapes
NX_BUILT = (32, 64, 128, 0)  # crm_kernel.h kNxBuilt (0: generic nx)
UNITS = {'crm_prep': ('crm_prep', ['-fmad=false']), 'crm_host': ('crm_host', []),
         'crm_serve': ('crm_serve', []), 'crm_tc_probe': ('crm_tc_probe', [])}
for _n in NX_BUILT:
    for _s in range(NUM_SHAPES):
        _d = ['-DCRM_INST_NX=%d' % _n, '-DCRM_INST_SHAPE=%d' % _s]
        UNITS['crm_fp64_nx%d_s%d' % (_n, _s)] = ('crm_columns', ['-fmad=false', '-DCRM_INST_T=double'] + _d)
        # FP32-mixed form: FP32 division and square root to the hardware's
        # approximate instructions (<= 2 ulp), denormals flushed; the FP64
        # parts of the form are unaffected by these flags
        UNITS['crm_fp32_nx%d_s%d' % (_n, _s)] = ('crm_columns', ['-DCRM_INST_T=float', '-prec-div=false',
                                                                 '-prec-sqrt=false', '-ftz=true'] + _d)
# 3D CRM: the generic kernel (nx, ny from the layout), launch shapes without
# shared-memory scratch planes only
SHAPES_3D = (0, 1, 3, 4)
for _s in SHAPES_3D:
    _d = ['-DCRM_INST_NX=0', '-DCRM_INST_NY=0', '-DCRM_INST_SHAPE=%d' % _s]
    UNITS['crm_fp64_3d_s%d' % _s] = ('crm_columns', ['-fmad=false', '-DCRM_INST_T=double'] + _d)
    UNITS['crm_fp32_3d_s%d' % _s] = ('crm_columns', ['-DCRM_INST_T=float', '-prec-div=false',
                                                     '-prec-sqrt=false', '-ftz=true'] + _d)
# the 3D FP32-mixed form with the tensor-core transforms (one launch shape,
# crm_kernel.h kTcShape)
UNITS['crm_fp32_3d_tc'] = ('crm_columns', ['-DCRM_INST_T=float', '-prec-div=false', '-prec-sqrt=false', '-ftz=true',
                                           '-DCRM_INST_NX=0', '-DCRM_INST_NY=0', '-DCRM_INST_SHAPE=4', '-DCRM_INST_VAR=1'])
# the FP64 form with multiply-add contraction (CRM_FP64_FMA): one launch
# shape each (crm_kernel.h kFmaShape2d, kFmaShape3d)
for _n in NX_BUILT:
    UNITS['crm_fp64fma_nx%d' % _n] = ('crm_columns', ['-DCRM_INST_T=double', '-DCRM_INST_NX=%d' % _n,
                                                      '-DCRM_INST_SHAPE=0', '-DCRM_INST_VAR=2'])
UNITS['crm_fp64fma_3d'] = ('crm_columns', ['-DCRM_INST_T=double', '-DCRM_INST_NX=0', '-DCRM_INST_NY=0',
                                           '-DCRM_INST_SHAPE=3', '-DCRM_INST_VAR=2'])


def _nvcc():
    for c in (os.environ.get('NVCC'), '/usr/local/cuda/bin/nvcc', 'nvcc'):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return 'nvcc'


def _sources():
    out = []
    for d in (CSRC, os.path.join(REPO, 'include')):
        out += [os.path.join(d, f) for f in os.listdir(d)
                if f.endswith(('.cu', '.cuh', '.h'))]
    return out


def up_to_date(lib=LIB):
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=False, phase_timers=False):
    """Compile the library if any source is newer than it; returns its path.
    phase_timers=True builds libcrm_gb300_prof.so, whose column kernel also
    accumulates clock64() cycles per phase (crm_debug_phase_cycles)."""
    lib = LIB_PROF if phase_timers else LIB
    if not force and up_to_date(lib):
        return lib
    odir = OBJ + ('_prof' if phase_timers else '')
    os.makedirs(odir, exist_ok=True)
    nvcc = _nvcc()
    extra = ['-DCRM_PHASE_TIMERS'] if phase_timers else []

    def compile_unit(name):
        obj = os.path.join(odir, name + '.o')
        src, flags = UNITS[name]
        cmd = [nvcc] + ARCH + COMMON + extra + flags + ['-c', os.path.join(CSRC, src + '.cu'), '-o', obj]
        if verbose:
            print(' '.join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed for %s:\n%s%s' % (name, r.stdout, r.stderr))
        return obj

    with ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = lib + '.tmp'
    cmd = [nvcc] + ARCH + ['-shared', '-o', tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('nvcc link failed:\n%s%s' % (r.stdout, r.stderr))
    os.replace(tmp, lib)
    return lib


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose=True, phase_timers='--phase-timers' in sys.argv))
