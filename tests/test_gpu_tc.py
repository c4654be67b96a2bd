"""The 3D pressure solve's x/y transforms on the tensor cores (tcgen05,
3xTF32; crm_debug_tc_transform) against the discrete Fourier transform in
fft991's coefficient order, and the FP32-mixed 3D form with them against the
same form with the warp FFT."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from crm_gb300 import synthetic as S
from crm_gb300 import crm_types as T
from crm_gb300.lib import CrmContext, load

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _probe(n, levels, direction):
    lib = load()
    f = lib.crm_debug_tc_transform
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    a = np.ascontiguousarray(levels, dtype=np.float32)
    out = np.zeros_like(a)
    rc = f(n, a.shape[0], direction, a.ctypes.data_as(C.POINTER(C.c_float)), out.ctypes.data_as(C.POINTER(C.c_float)))
    assert rc == T.CRM_OK, rc
    return out


def _matrices(n):
    i = np.arange(n)
    bf = np.zeros((n + 2, n))
    bi = np.zeros((n, n + 2))
    for k in range(n // 2 + 1):
        th = 2 * np.pi * i * k / n
        w = 1.0 if k in (0, n // 2) else 2.0
        bf[2 * k], bi[:, 2 * k] = np.cos(th) / n, w * np.cos(th)
        if 0 < k < n // 2:
            bf[2 * k + 1], bi[:, 2 * k + 1] = -np.sin(th) / n, -w * np.sin(th)
    return bf, bi


@pytest.mark.parametrize('n,nlev', [(32, 9), (16, 9), (32, 58)])
def test_forward_is_the_2d_real_transform(gpu_lib, n, nlev):
    """Rows j = 1..n, columns i = 1..n of each level in; F = Bf P Bf^T out in
    columns 1..n+1 and rows 1..n+2 (levels beyond a whole tile included)."""
    rng = np.random.default_rng(n + nlev)
    ff = rng.standard_normal((nlev, n + 2, n + 2)).astype(np.float32)
    out = _probe(n, ff, -1)
    bf, _ = _matrices(n)
    for k in range(nlev):
        want = bf @ ff[k, :n, :n].astype(np.float64) @ bf.T          # [jj][c]
        got = out[k, :, :n + 1]
        err = np.max(np.abs(got - want[:, :n + 1])) / np.max(np.abs(want))
        assert err < 2e-6, (k, err)


@pytest.mark.parametrize('n', [16, 32])
def test_forward_matches_fft991_rows_then_columns(gpu_lib, n):
    """The same coefficients as the reference's transform order: fft991 on
    every row, then on every x coefficient's column."""
    rng = np.random.default_rng(7 + n)
    p = rng.standard_normal((n, n))
    ff = np.zeros((1, n + 2, n + 2), dtype=np.float32)
    ff[0, :n, :n] = p
    out = _probe(n, ff, -1)
    g = np.zeros((n + 2, n + 2))
    for j in range(n):
        a = np.zeros(n + 2)
        a[:n] = p[j]
        g[j] = oracle.fft991(a, -1)
    for c in range(n + 1):
        g[:, c] = oracle.fft991(g[:, c].copy(), -1)
    err = np.max(np.abs(out[0, :, :n + 1] - g[:, :n + 1])) / np.max(np.abs(g))
    assert err < 5e-6, err


@pytest.mark.parametrize('n,nlev', [(32, 9), (16, 9)])
def test_inverse_and_round_trip(gpu_lib, n, nlev):
    rng = np.random.default_rng(100 + n)
    _, bi = _matrices(n)
    ff = rng.standard_normal((nlev, n + 2, n + 2)).astype(np.float32)
    out = _probe(n, ff, +1)
    for k in range(nlev):
        f = ff[k].astype(np.float64).copy()
        f[:, n + 1] = 0.0                      # Im X_n/2 is not read
        want = bi @ f @ bi.T
        err = np.max(np.abs(out[k, :n, :n] - want)) / np.max(np.abs(want))
        assert err < 2e-6, (k, err)
    p = np.zeros((nlev, n + 2, n + 2), dtype=np.float32)
    p[:, :n, :n] = rng.standard_normal((nlev, n, n))
    back = _probe(n, _probe(n, p, -1), +1)
    assert np.max(np.abs(back[:, :n, :n] - p[:, :n, :n])) < 2e-6 * np.max(np.abs(p))


@pytest.mark.parametrize('n,moist,dt_gl', [(32, True, 300.0), (16, False, 600.0)])
def test_fp32_3d_tensor_core_transforms_against_the_fft(gpu_lib, n, moist, dt_gl):
    """The FP32-mixed 3D form with the tensor-core transforms
    (CRM_GB300_TRANSFORM=tc, its own kernel instance) and with the warp FFT
    (the default): both within the form's 1e-4 tendency target against the
    FP64 form, and close to each other."""
    cfg, cin, st, rad, desc = S.workload_3d(ncrms=2, nx=n, ny=n, moist=moist)
    desc.dt_gl = dt_gl
    res = {}
    for mode in ('tc', 'fft'):
        if mode == 'tc':
            os.environ['CRM_GB300_TRANSFORM'] = 'tc'
        try:
            c = T.CrmConfig(**{**cfg.__dict__, 'precision': T.CRM_FP32_MIXED, 'max_ncrms': desc.ld})
            ctx = CrmContext(c)
            out = T.CrmOutput(desc.ld, c.crm_nx, c.crm_ny, c.crm_nz, c.plev)
            s2 = st.copy()
            ctx.run(desc, cin, s2, rad.copy(), out, raise_on_error=True)
            res[mode] = (s2, out)
        finally:
            os.environ.pop('CRM_GB300_TRANSFORM', None)
    c64 = T.CrmConfig(**{**cfg.__dict__, 'precision': T.CRM_FP64, 'max_ncrms': desc.ld})
    out64 = T.CrmOutput(desc.ld, c64.crm_nx, c64.crm_ny, c64.crm_nz, c64.plev)
    s64 = st.copy()
    CrmContext(c64).run(desc, cin, s64, rad.copy(), out64, raise_on_error=True)
    for mode, (s2, out) in res.items():
        e = {k: rel_l2(getattr(out, k), getattr(out64, k)) for k in ('sltend', 'qltend')}
        e['w'] = rel_l2(s2.w_wind, s64.w_wind)
        e['t'] = rel_l2(s2.temperature, s64.temperature)
        print('3D %dx%d FP32-mixed (%s transforms) vs FP64:' % (n, n, mode), e)
        assert e['sltend'] <= 1e-4 and e['qltend'] <= 1e-4 and e['w'] <= 5e-3 and e['t'] <= 1e-6, (mode, e)
    d = rel_l2(res['tc'][0].w_wind, res['fft'][0].w_wind)
    assert d <= 5e-3, d
