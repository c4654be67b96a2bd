"""Launch shapes and the autotuner: every launchable shape gives the same
bits in the FP64 form (compiled without multiply-add contraction) and the
same result to FP32 rounding in the FP32-mixed form (the compiler contracts
multiply-adds per kernel instance), and autotune() leaves the handle on the
fastest shape with the batch state restored."""
import numpy as np
import pytest

from crm_gb300 import crm_types as T
from crm_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('precision', [T.CRM_FP64, T.CRM_FP32_MIXED])
def test_shapes_agree_and_autotune(gpu_lib, precision):
    import torch
    from crm_gb300.autotune import autotune, shapes
    from crm_gb300.device import DeviceCrmArrays
    from crm_gb300.lib import CrmContext
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=24, moist=True, precision=precision)
    desc.dt_gl = 100.0
    cfg.max_ncrms = 24
    ctx = CrmContext(cfg)
    dev = DeviceCrmArrays(cfg, cin, st, rad, desc, desc._keep)
    stream = torch.cuda.current_stream().cuda_stream
    ref = None
    ran = 0
    for s, _, _, _ in shapes():
        if ctx.set_launch_shape(s) != 0:
            continue
        dev.reset_state(st)
        ctx.run_device(dev, stream)
        torch.cuda.synchronize()
        got = {n: dev.state_numpy(n) for n in T.STATE_FIELDS}
        got['sltend'] = dev.out_numpy('sltend')
        if ref is None:
            ref = got
        elif precision == T.CRM_FP64:
            for n in ref:
                assert np.array_equal(ref[n], got[n]), (s, n)
        else:
            for n in ('temperature', 'qt', 'u_wind'):
                a, b = ref[n].ravel(), got[n].ravel()
                assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(a), (s, n)
        ran += 1
    assert ran >= 2
    assert ctx.set_launch_shape(99) == T.CRM_ERR_ARG
    best, times = autotune(ctx, dev, st)
    assert best in times and ctx.launch_shape == best
    assert np.array_equal(dev.state_numpy('temperature'), np.asfortranarray(st.temperature))
