"""The 3D CRM (crm_ny > 1) on the device against the CPU restatement.

FP64 plain form: bit-exact, as for the 2D CRM (the same operations in the
same order: MPDATA and SGS fluxes in x and y, the x-then-y real transforms of
the pressure solve, horizontal sums in the reference's (j, i) loop order).
FP32-mixed form: relative L2 bounds after one GCM step.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from crm_gb300 import synthetic as S
from crm_gb300 import crm_types as T
from crm_gb300.lib import CrmContext, load

from conftest import rel_l2
from test_gpu_parity import mismatches, run_both

pytestmark = pytest.mark.gpu


def test_fp64_bitexact_3d_16x16(gpu_lib):
    cfg, cin, st, rad, desc = S.workload_3d(ncrms=2, nx=16, ny=16)
    desc.dt_gl = 100.0
    assert mismatches(*run_both(cfg, cin, st, rad, desc)) == []


def test_fp64_bitexact_3d_32x32(gpu_lib):
    cfg, cin, st, rad, desc = S.workload_3d(ncrms=2)
    desc.dt_gl = 200.0
    assert mismatches(*run_both(cfg, cin, st, rad, desc)) == []


def test_fp64_bitexact_3d_rectangular(gpu_lib):
    """nx != ny and dy != dx: the y transform, the (i, j) eigenvalues and
    the y metric terms each have their own sizes."""
    cfg, cin, st, rad, desc = S.workload_3d(ncrms=2, nx=32, ny=16)
    cfg.crm_dy = 1500.0
    desc.dt_gl = 100.0
    assert mismatches(*run_both(cfg, cin, st, rad, desc)) == []


def test_fp64_bitexact_3d_moist(gpu_lib):
    """Saturated layers and falling precipitation in 3D."""
    cfg, cin, st, rad, desc = S.workload_3d(ncrms=2, nx=16, ny=16, moist=True)
    desc.dt_gl = 600.0
    a, b = run_both(cfg, cin, st, rad, desc)
    assert a[2].cltot.max() > 0 and a[2].precc.max() > 0
    assert mismatches(a, b) == []


def test_fp64_bitexact_3d_reference_batch(gpu_lib):
    """CRM_REFERENCE_BATCH in 3D: the grid-wide CFL maxima couple the columns."""
    cfg, cin, st, rad, desc = S.workload_3d(ncrms=3, nx=16, ny=16, batch_mode=T.CRM_REFERENCE_BATCH)
    desc.dt_gl = 100.0
    st.w_wind[1, :, :, 10] = 30.0
    assert mismatches(*run_both(cfg, cin, st, rad, desc)) == []


# relative L2 bounds of the FP32-mixed form after one 3D GCM step of 600 s
# (measured dry / moist: temperature 7.6e-8 / 2.6e-7, qt 1.1e-6 / 3.1e-6,
# u 1.6e-6 / 8.1e-6, v 2.9e-6 / 1.6e-5, w 6.7e-4 / 1.2e-3, sltend 9.2e-5 /
# 9.2e-5, qltend 2.6e-5 / 5.8e-6, tk 3.0e-4 / 1.2e-3); the GCM tendencies
# are held to the 1e-4 target
BOUNDS_3D = {'temperature': 1e-6, 'qt': 2e-5, 'u_wind': 1e-4, 'v_wind': 1e-4, 'w_wind': 5e-3,
             'sltend': 1e-4, 'qltend': 1e-4, 'qcltend': 1e-4, 'qiltend': 1e-4}
OUTPUT_BOUND_3D = 3e-2


@pytest.mark.parametrize('moist', [False, True])
def test_fp32_mixed_3d(gpu_lib, moist):
    cfg, cin, st, rad, desc = S.workload_3d(ncrms=2, nx=16, ny=16, moist=moist)
    desc.dt_gl = 600.0
    st_o, rad_o = st.copy(), rad.copy()
    rc, _, out_o = oracle.run(cfg, desc, cin, st_o, rad_o)
    assert rc == 0
    cfg.precision = T.CRM_FP32_MIXED
    cfg.max_ncrms = desc.ld
    ctx = CrmContext(cfg)
    out_g = T.CrmOutput(desc.ld, cfg.crm_nx, cfg.crm_ny, cfg.crm_nz, cfg.plev)
    st_g, rad_g = st.copy(), rad.copy()
    ctx.run(desc, cin, st_g, rad_g, out_g, raise_on_error=True)
    e = {n: rel_l2(getattr(st_g, n), getattr(st_o, n)) for n in ('temperature', 'qt', 'u_wind', 'v_wind', 'w_wind')}
    for n, a in out_g.arrays().items():
        assert np.isfinite(a).all(), n
        e[n] = rel_l2(a, getattr(out_o, n))
    print('fp32-mixed rel-L2 vs fp64 oracle (3D 16x16x58, moist=%s):' % moist, e)
    for n, bound in BOUNDS_3D.items():
        assert e[n] <= bound, (n, e[n], bound)
    for n, v in e.items():
        assert v <= OUTPUT_BOUND_3D, (n, v)


def _create_status(cfg):
    lib = load()
    st = C.c_int(0)
    c_cfg = cfg.to_c()
    h = lib.crm_create(C.byref(c_cfg), C.byref(st))
    if h:
        lib.crm_destroy(h)
    return st.value


def test_3d_configurations_not_built(gpu_lib):
    """3D radiation groups coarser than the CRM grid and transform lengths
    with factors other than 2 and 4 are refused with CRM_ERR_UNSUPPORTED;
    the fixed-scratch entry takes 2D only."""
    cfg = S.config_3d(nx=16, ny=16)
    cfg.max_ncrms = 2
    assert _create_status(cfg) == T.CRM_OK
    coarse = S.config_3d(nx=16, ny=16)
    coarse.crm_nx_rad, coarse.crm_ny_rad, coarse.max_ncrms = 8, 8, 2
    assert _create_status(coarse) == T.CRM_ERR_UNSUPPORTED
    odd = S.config_3d(nx=16, ny=24)
    odd.max_ncrms = 2
    assert _create_status(odd) == T.CRM_ERR_UNSUPPORTED
    small = S.config_3d(nx=16, ny=4)
    small.max_ncrms = 2
    assert _create_status(small) == T.CRM_ERR_ARG
