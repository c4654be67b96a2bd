"""Accuracy of the deterministic exp/log/pow/atan (include/crm_detmath.h).

Both the CPU oracle and the FP64 device form evaluate these functions with
the same source, which is what makes the two bit-identical; here the host
build is compared with the platform libm (Python's math module) over the
argument ranges the CRM uses.  Bounds: exp, log, pow <= 2 ulp; atan <= 4 ulp.
"""
import ctypes as C
import math
import os
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include "crm_detmath.h"
using namespace crm_detmath;
extern "C" {
void v_exp(const double *x, double *y, int n) { for (int i = 0; i < n; ++i) y[i] = det_exp(x[i]); }
void v_log(const double *x, double *y, int n) { for (int i = 0; i < n; ++i) y[i] = det_log(x[i]); }
void v_atan(const double *x, double *y, int n) { for (int i = 0; i < n; ++i) y[i] = det_atan(x[i]); }
void v_pow(const double *x, const double *e, double *y, int n) {
  for (int i = 0; i < n; ++i) y[i] = det_pow(x[i], e[i]);
}
}
'''


@pytest.fixture(scope='module')
def dm(tmp_path_factory):
    d = tmp_path_factory.mktemp('detmath')
    src = d / 'dm.cpp'
    src.write_text(SRC)
    so = d / 'libdm.so'
    subprocess.check_call(['g++', '-O2', '-std=c++17', '-ffp-contract=off', '-fPIC', '-shared',
                           '-I', os.path.join(REPO, 'include'), '-o', str(so), str(src)])
    lib = C.CDLL(str(so))
    P = C.POINTER(C.c_double)
    for n in ('v_exp', 'v_log', 'v_atan'):
        getattr(lib, n).argtypes = [P, P, C.c_int]
    lib.v_pow.argtypes = [P, P, P, C.c_int]
    return lib


def _call(fn, *xs):
    xs = [np.ascontiguousarray(x, dtype=np.float64) for x in xs]
    y = np.empty_like(xs[0])
    P = C.POINTER(C.c_double)
    fn(*[x.ctypes.data_as(P) for x in xs], y.ctypes.data_as(P), len(y))
    return y


def ulps(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    ia = a.view(np.int64).astype(object)
    ib = b.view(np.int64).astype(object)
    # map to a monotonic integer line
    fa = [x if x >= 0 else -(x & 0x7FFFFFFFFFFFFFFF) for x in ia]
    fb = [x if x >= 0 else -(x & 0x7FFFFFFFFFFFFFFF) for x in ib]
    return max(abs(x - y) for x, y in zip(fa, fb))


RNG = np.random.Generator(np.random.PCG64(7))


def test_exp(dm):
    x = np.concatenate([RNG.uniform(-50, 50, 4000), RNG.uniform(-1, 1, 2000),
                        RNG.uniform(-700, 700, 1000), [0.0, 1e-300, -1e-300, 1.0, -1.0]])
    y = _call(dm.v_exp, x)
    ref = np.array([math.exp(v) for v in x])
    assert ulps(y, ref) <= 2


def test_log(dm):
    x = np.concatenate([10.0 ** RNG.uniform(-30, 6, 4000), RNG.uniform(0.5, 2.0, 2000),
                        [1.0, 2.0, 0.5, 1e-300, 1e300, 1 - 1e-12, 1 + 1e-12]])
    y = _call(dm.v_log, x)
    ref = np.array([math.log(v) for v in x])
    assert ulps(y, ref) <= 2


def test_pow(dm):
    # bases: densities, mixing ratios, pressure ratios, slopes; exponents of
    # the sam1mom rates (0.8, 0.25, 0.5, (3+b)/4 ...) and general ones
    x = np.concatenate([10.0 ** RNG.uniform(-8, 4, 3000), RNG.uniform(0.1, 3.0, 2000)])
    e = np.concatenate([RNG.choice([0.8, 0.25, 0.5, 0.2, 0.4, 0.525, 0.6875, 0.8125,
                                    1.0 / 3.0, 1.5, 2.0, -0.5], 3000),
                        RNG.uniform(-3, 3, 2000)])
    y = _call(dm.v_pow, x, e)
    ref = np.array([math.pow(a, b) for a, b in zip(x, e)])
    assert ulps(y, ref) <= 2
    assert _call(dm.v_pow, np.array([0.0]), np.array([0.5]))[0] == 0.0
    assert _call(dm.v_pow, np.array([3.0]), np.array([0.0]))[0] == 1.0


def test_atan(dm):
    x = np.concatenate([RNG.uniform(-1, 1, 3000), 10.0 ** RNG.uniform(-6, 6, 3000),
                        -(10.0 ** RNG.uniform(-6, 6, 1000)), [0.0, 1.0, -1.0, 0.2679491924311227]])
    y = _call(dm.v_atan, x)
    ref = np.array([math.atan(v) for v in x])
    assert ulps(y, ref) <= 4
