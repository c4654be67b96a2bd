"""crm_run_device and crm_run_device_noalloc recorded into a CUDA graph.

A GCM that keeps its physics on the GPU captures its step once and replays
it.  Both device entry points enqueue only kernel launches (and event
records) on the caller's stream, so they can be captured; a replay must give
the same bits as a direct call on the same inputs, and a second replay the
same again (nothing of the first replay's state leaks into the next).
"""
import numpy as np
import pytest

from crm_gb300 import crm_types as T
from crm_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _snapshot(dev):
    return {g + '.' + n: t.cpu().numpy().copy()
            for g in ('state', 'rad', 'out') for n, t in getattr(dev, g).items()}


def _same(a, b):
    return [n for n in a if not np.array_equal(a[n], b[n])]


def _run_graph(gpu_lib, prec, noalloc):
    import torch
    from crm_gb300.device import DeviceCrmArrays
    from crm_gb300.lib import CrmContext, run_device_noalloc
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=8, moist=True)
    desc.dt_gl = 200.0
    cfg.precision = prec
    cfg.max_ncrms = desc.ld
    ctx = None if noalloc else CrmContext(cfg)
    dev = DeviceCrmArrays(cfg, cin, st, rad, desc, desc._keep)

    def call(stream):
        if noalloc:
            rc = run_device_noalloc(cfg, dev, stream)
            assert rc == T.CRM_OK, gpu_lib.crm_status_string(rc)
        else:
            ctx.run_device(dev, stream)

    # direct call (also the no-allocation entry's per-device set-up, which
    # has to happen outside a capture)
    call(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert int(dev.status.abs().sum().item()) == 0
    ref = _snapshot(dev)

    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    dev.reset_state(st)
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=side):
        call(side.cuda_stream)
    for rep in range(2):
        dev.reset_state(st)
        dev.out['precc'].fill_(-1.0)            # replay must rewrite the outputs
        graph.replay()
        torch.cuda.synchronize()
        assert int(dev.status.abs().sum().item()) == 0
        bad = _same(ref, _snapshot(dev))
        assert not bad, (rep, bad[:8])
    if ctx is not None:
        ctx.close()


@pytest.mark.parametrize('prec', [T.CRM_FP64, T.CRM_FP32_MIXED])
def test_graph_replay_run_device(gpu_lib, prec):
    _run_graph(gpu_lib, prec, noalloc=False)


@pytest.mark.parametrize('prec', [T.CRM_FP64, T.CRM_FP32_MIXED])
def test_graph_replay_run_device_noalloc(gpu_lib, prec):
    _run_graph(gpu_lib, prec, noalloc=True)
