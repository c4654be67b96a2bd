"""crm_run_device_noalloc against crm_run_device, through the C ABI.

The no-allocation entry point runs the same kernels with their scratch in the
library's fixed static device array (fewer CTAs, columns looped over them).
Each column's result depends only on that column, so both entry points must
agree bit for bit (the tolerance of the FP64 parity tests, zero); the FP32
case is held to the same zero tolerance.  Two calls in a row check that the
shared scratch keeps no state from one call to the next that changes results.

The file name makes pytest collect it last; it also passes alone in a fresh
process (the first call performs the per-device set-up).
"""
import numpy as np
import pytest

from crm_gb300 import crm_types as T
from crm_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _compare(a, b):
    bad = []
    for group in ('state', 'rad', 'out'):
        da, db = getattr(a, group), getattr(b, group)
        for n in da:
            x, y = da[n].cpu().numpy(), db[n].cpu().numpy()
            if not np.array_equal(x, y):
                bad.append((group + '.' + n, float(np.max(np.abs(x - y)))))
    return bad


def _pair(gpu_lib, cfg, cin, st, rad, desc, calls=2):
    import torch
    from crm_gb300.device import DeviceCrmArrays
    from crm_gb300.lib import CrmContext, run_device_noalloc
    cfg.max_ncrms = max(cfg.max_ncrms, desc.ld)
    ctx = CrmContext(cfg)
    a = DeviceCrmArrays(cfg, cin, st, rad, desc, desc._keep)
    b = DeviceCrmArrays(cfg, cin, st, rad, desc, desc._keep)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(calls):
        ctx.run_device(a, stream)
        rc = run_device_noalloc(cfg, b, stream)
        assert rc == T.CRM_OK, gpu_lib.crm_status_string(rc)
        torch.cuda.synchronize()
        assert int(a.status.abs().sum().item()) == 0
        assert torch.equal(a.status, b.status)
        bad = _compare(a, b)
        assert not bad, (call, bad[:8])
    ctx.close()


def test_noalloc_matches_fp64_32x28(gpu_lib):
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=16, moist=True)
    desc.dt_gl = 200.0
    _pair(gpu_lib, cfg, cin, st, rad, desc)


def test_noalloc_matches_fp64_64x58_looped(gpu_lib):
    # 48 columns of 64 x 58 in FP64 need about 68 MB of slabs: the 32 MiB
    # scratch holds 21, so each CTA runs two or three columns in turn.
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=48, moist=True)
    desc.dt_gl = 100.0
    _pair(gpu_lib, cfg, cin, st, rad, desc)


def test_noalloc_matches_fp32_64x58(gpu_lib):
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=64, precision=T.CRM_FP32_MIXED)
    desc.dt_gl = 100.0
    _pair(gpu_lib, cfg, cin, st, rad, desc)


def test_noalloc_rejects_oversize(gpu_lib):
    import ctypes as C
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=4)
    # 100000 columns of set-up values alone (257 MB) exceed the scratch; the
    # size check runs before any device work and before the array pointers
    # are looked at, so empty argument structs are enough here.
    d = T.CCrmCallDesc(0, 100000, 100000, 100.0, 2, None)
    rc = gpu_lib.crm_run_device_noalloc(C.byref(cfg.to_c()), C.byref(d), C.byref(T.CCrmInput()),
                                        C.byref(T.CCrmState()), C.byref(T.CCrmRad()),
                                        C.byref(T.CCrmOutput()), None, None)
    assert rc == T.CRM_ERR_TOO_LARGE
    big = S.config_64x58(nx=2048)
    d = T.CCrmCallDesc(0, 1, 1, 100.0, 2, None)
    rc = gpu_lib.crm_run_device_noalloc(C.byref(big.to_c()), C.byref(d), C.byref(T.CCrmInput()),
                                        C.byref(T.CCrmState()), C.byref(T.CCrmRad()),
                                        C.byref(T.CCrmOutput()), None, None)
    assert rc == T.CRM_ERR_TOO_LARGE
