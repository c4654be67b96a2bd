"""The serving loop on the GPU: a chunk's results are the same alone and in
a mix of concurrent chunks of other sizes (continuous batching over resident
slots), and they equal a direct crm_run of the same columns."""
import numpy as np
import pytest

from crm_gb300 import crm_types as T
from crm_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

DT_GL = 300.0


def _configs():
    return [T.CrmConfig(crm_nx=nx, crm_ny=1, crm_nz=nz, plev=72, crm_dx=1000.0, crm_dt=10.0,
                        precision=T.CRM_FP32_MIXED) for nx, nz in ((32, 28), (64, 58))]


def _chunk(cfg, ncol, gcol0, seed):
    from crm_gb300.serve_bench import make_chunk
    return make_chunk(cfg, ncol, gcol0, seed)


def _drive(server, cfg, chunk, steps):
    from crm_gb300.serving import apply_tendencies
    cin, st, rad, gcol = chunk
    cin = cin.copy()
    ch = server.open_chunk(cfg, cin, st, rad, gcol)
    res = []
    for _ in range(steps):
        vals, status = server.step(ch, cin, DT_GL).result(timeout=120)
        assert not status.any()
        res.append(vals)
        apply_tendencies(cin, vals, DT_GL)
    server.close_chunk(ch)
    return res


def test_chunk_alone_equals_chunk_in_mix(gpu_lib):
    import threading
    from crm_gb300.serving import CrmServer
    cfgs = _configs()
    a = _chunk(cfgs[1], 5, 101, seed=7)
    server = CrmServer(cfgs, capacity=256)
    alone = _drive(server, cfgs[1], a, 3)
    # the same chunk again, now with four others of both sizes in flight
    others = [(cfgs[i % 2], _chunk(cfgs[i % 2], 3 + 7 * i, 1000 * (i + 1), seed=i)) for i in range(4)]
    out = {}
    ts = [threading.Thread(target=lambda c=c, ch=ch, i=i: out.__setitem__(i, _drive(server, c, ch, 3)))
          for i, (c, ch) in enumerate(others)]
    for t in ts:
        t.start()
    mixed = _drive(server, cfgs[1], a, 3)
    for t in ts:
        t.join()
    server.close()
    assert len(out) == 4
    assert server.launches >= 3
    for s in range(3):
        for n, v in alone[s].items():
            assert np.array_equal(v, mixed[s][n]), (s, n)


def test_serving_step_equals_crm_run(gpu_lib):
    """First step of a chunk through the server == crm_run of the same columns."""
    from crm_gb300.lib import CrmContext
    from crm_gb300.serving import CrmServer
    cfg = _configs()[0]
    cin, st, rad, gcol = _chunk(cfg, 6, 11, seed=3)
    server = CrmServer([cfg], capacity=64)
    vals = _drive(server, cfg, (cin, st, rad, gcol), 1)[0]
    server.close()
    c2 = T.CrmConfig(**{**cfg.__dict__, 'max_ncrms': 6})
    ctx = CrmContext(c2)
    out = T.CrmOutput(6, cfg.crm_nx, 1, cfg.crm_nz, cfg.plev)
    desc = T.call_desc(6, 6, DT_GL, 1, gcol)
    status = ctx.run(desc, cin, st.copy(), rad.copy(), out)
    assert not status.any()
    for n, v in vals.items():
        assert np.array_equal(v, getattr(out, n)), n


def test_checkpoint_and_restore_chunk(gpu_lib, tmp_path):
    """Two steps in one server == one step, checkpoint, a new server restored
    from the file, second step."""
    from crm_gb300.serving import CrmServer, apply_tendencies
    cfg = _configs()[0]
    cin, st, rad, gcol = _chunk(cfg, 4, 21, seed=5)
    server = CrmServer([cfg], capacity=32)
    ref = _drive(server, cfg, (cin, st, rad, gcol), 2)
    server.close()

    server = CrmServer([cfg], capacity=32)
    cin1 = cin.copy()
    ch = server.open_chunk(cfg, cin1, st, rad, gcol)
    vals, status = server.step(ch, cin1, DT_GL).result(timeout=120)
    assert not status.any()
    apply_tendencies(cin1, vals, DT_GL)
    p = str(tmp_path / 'chunk.ckpt')
    server.checkpoint_chunk(ch, p)
    server.close_chunk(ch)
    server.close()

    server = CrmServer([cfg], capacity=32)
    ch = server.restore_chunk(p, cin1)
    vals2, status = server.step(ch, cin1, DT_GL).result(timeout=120)
    server.close()
    assert not status.any()
    for n, v in ref[1].items():
        assert np.array_equal(v, vals2[n]), n


def test_resume_chunk_from_a_gcm_restart_file(gpu_lib, tmp_path):
    """Two steps in one server == one step, the chunk's state written in the
    GCM restart file's layout (CRM_* on a 64-column grid), a new server
    resuming the chunk from that file, second step."""
    from crm_gb300.serving import CrmServer, apply_tendencies
    cfg = _configs()[1]
    cin, st, rad, gcol = _chunk(cfg, 4, 30, seed=6)
    server = CrmServer([cfg], capacity=32)
    ref = _drive(server, cfg, (cin, st, rad, gcol), 2)
    server.close()

    server = CrmServer([cfg], capacity=32)
    cin1 = cin.copy()
    ch = server.open_chunk(cfg, cin1, st, rad, gcol)
    vals, status = server.step(ch, cin1, DT_GL).result(timeout=120)
    assert not status.any()
    apply_tendencies(cin1, vals, DT_GL)
    p = str(tmp_path / 'gcm_restart.nc')
    server.write_gcm_restart(ch, p, ncol=64)
    server.close_chunk(ch)
    server.close()

    server = CrmServer([cfg], capacity=32)
    ch = server.restore_chunk_from_gcm_restart(p, cfg, gcol, cin1)
    vals2, status = server.step(ch, cin1, DT_GL).result(timeout=120)
    server.close()
    assert not status.any()
    for n, v in ref[1].items():
        assert np.array_equal(v, vals2[n]), n


def test_two_steps_of_one_chunk_submitted_back_to_back(gpu_lib):
    """A chunk's second request, submitted before its first completes, waits
    for it: the results equal the two steps run one after the other."""
    from crm_gb300.serving import CrmServer
    cfg = _configs()[0]
    cin, st, rad, gcol = _chunk(cfg, 5, 31, seed=9)
    server = CrmServer([cfg], capacity=32)
    ch = server.open_chunk(cfg, cin, st, rad, gcol)
    seq = []
    for _ in range(2):
        vals, status = server.step(ch, cin, DT_GL).result(timeout=120)
        assert not status.any()
        seq.append(vals)
    server.close_chunk(ch)
    ch = server.open_chunk(cfg, cin, st, rad, gcol)
    f1 = server.step(ch, cin, DT_GL)
    f2 = server.step(ch, cin, DT_GL)
    both = [f1.result(timeout=120), f2.result(timeout=120)]
    server.close()
    assert ch.steps == 2
    for s in range(2):
        assert not both[s][1].any()
        for n, v in seq[s].items():
            assert np.array_equal(v, both[s][0][n]), (s, n)
    # the second step differs from the first (it continued the state)
    assert not np.array_equal(seq[0]['sltend'], seq[1]['sltend'])


def test_pool_is_charged_to_the_budget(gpu_lib):
    """A pool's device memory is charged when it is created: a budget that
    cannot hold any pool of the configuration refuses the chunk with
    CRM_ERR_BUDGET, one that holds part of a full pool gets a smaller pool,
    and closing the server's chunks lets another configuration take the
    memory of an idle pool."""
    from crm_gb300.lib import plan_device_bytes
    from crm_gb300.serving import BudgetError, CrmServer, pool_bytes
    cfgs = _configs()
    cfg = cfgs[0]
    cin, st, rad, gcol = _chunk(cfg, 4, 41, seed=2)
    hb = lambda cap: plan_device_bytes(T.CrmConfig(**{**cfg.__dict__, 'max_ncrms': cap}))
    full = pool_bytes(cfg, 256, 3, hb)
    small = pool_bytes(cfg, 4, 3, hb)
    server = CrmServer(cfgs, capacity=256, hbm_budget=small - 1)
    with pytest.raises(BudgetError) as e:
        server.open_chunk(cfg, cin, st, rad, gcol)
    assert e.value.status == T.CRM_ERR_BUDGET
    server.close()
    # room for a small pool of each configuration, not for both at once
    c1 = cfgs[1]
    hb1 = lambda cap: plan_device_bytes(T.CrmConfig(**{**c1.__dict__, 'max_ncrms': cap}))
    small1 = pool_bytes(c1, 4, 3, hb1)
    assert small + small1 - 1 < full
    server = CrmServer(cfgs, capacity=256, hbm_budget=small + small1 - 1)
    ch = server.open_chunk(cfg, cin, st, rad, gcol)
    pool = server.pools[ch.key]
    assert 4 <= pool.capacity < 256
    assert server.budget.used == server.pool_charge[ch.key] <= server.budget.total
    held = sum(c.device_bytes for c in pool.ctx)
    assert held <= server.pool_charge[ch.key]
    server.close_chunk(ch)
    # the other configuration needs the memory: the idle pool is released
    cin1, st1, rad1, gcol1 = _chunk(c1, 4, 51, seed=3)
    ch1 = server.open_chunk(c1, cin1, st1, rad1, gcol1)
    assert ch.key not in server.pools and ch1.key in server.pools
    assert server.budget.used == server.pool_charge[ch1.key]
    server.close_chunk(ch1)
    server.close()
