"""Host logic of the serving loop (no GPU): slot pools, HBM admission
budget, per-slot sizes, and applying the CRM tendencies to GCM columns."""
import threading

import numpy as np
import pytest

from crm_gb300 import synthetic as S
from crm_gb300.serving import HbmBudget, SlotPool, apply_tendencies, slot_bytes


def test_slot_pool_alloc_free():
    p = SlotPool(10)
    a = p.alloc(4)
    b = p.alloc(6)
    assert sorted(a + b) == list(range(10))
    assert p.alloc(1) is None
    p.free(a)
    assert p.available == 4
    with pytest.raises(ValueError):
        p.free(a[:1])
    c = p.alloc(4)
    assert sorted(c) == sorted(a)


def test_slot_pool_threads_never_share_a_slot():
    p = SlotPool(64)
    got = []
    lock = threading.Lock()

    def worker():
        for _ in range(200):
            s = p.alloc(3)
            if s is None:
                continue
            with lock:
                got.append(tuple(s))
                assert len(set(sum(got, ()))) == 3 * len(got)
                got.remove(tuple(s))
            p.free(s)

    ts = [threading.Thread(target=worker) for _ in range(8)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert p.available == 64


def test_hbm_budget():
    b = HbmBudget(100)
    assert b.reserve(60)
    assert not b.reserve(41)
    assert b.reserve(40)
    b.release(100)
    assert b.used == 0
    with pytest.raises(ValueError):
        b.release(1)


def test_slot_bytes_scale():
    small = slot_bytes(S.config_64x58(nx=32))
    big = slot_bytes(S.config_64x58(nx=128))
    assert 3.5 < big / small < 4.1
    # 120 GB holds ~10^5 columns of 128 x 58
    assert 120 * 2 ** 30 // big > 50_000


def test_apply_tendencies():
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=3)
    t0, q0 = cin.tl.copy(), cin.ql.copy()
    vals = {'sltend': np.full((3, cfg.plev), 1004.64), 'qltend': np.full((3, cfg.plev), -1e-9),
            'qcltend': np.zeros((3, cfg.plev)), 'qiltend': np.zeros((3, cfg.plev))}
    apply_tendencies(cin, vals, 10.0)
    assert np.allclose(cin.tl - t0, 10.0)
    assert np.all(cin.ql >= 0) and np.allclose(cin.ql, np.maximum(q0 - 1e-8, 0))


def test_config_key_groups_by_physics_not_capacity():
    from crm_gb300 import crm_types as T
    from crm_gb300.serving import config_key
    a = S.config_64x58()
    b = S.config_64x58()
    b.max_ncrms = 4096                                   # capacity only
    assert config_key(a) == config_key(b)
    for change in ({'crm_nx': 32}, {'crm_nz': 28}, {'precision': T.CRM_FP32_MIXED},
                   {'use_crm_accel': 1}, {'crm_dt': 20.0}, {'batch_mode': T.CRM_REFERENCE_BATCH}):
        c = T.CrmConfig(**{**a.__dict__, **change})
        assert config_key(c) != config_key(a), change


def test_select_launch_one_request_per_chunk():
    """A launch takes at most one request per chunk and none of a chunk with
    a step in flight; requests with another (dt_gl, first-step) tag wait."""
    from crm_gb300.serving import Chunk, StepRequest, select_launch
    a, b, c = (Chunk(('k',), [i], [i], 8) for i in range(3))
    b.steps = 1
    rs = [StepRequest(a, None, 300.0), StepRequest(a, None, 300.0), StepRequest(c, None, 300.0),
          StepRequest(b, None, 300.0), StepRequest(c, None, 600.0)]
    take, rest = select_launch(rs, busy=set())
    assert [r.chunk for r in take] == [a, c]
    assert rest == [rs[1], rs[3], rs[4]]
    take, rest = select_launch(rs, busy={id(a)})
    assert [r.chunk for r in take] == [c]
    take, rest = select_launch([rs[1], rs[3]], busy={id(a)})
    assert [r.chunk for r in take] == [b] and rest == [rs[1]]
    take, rest = select_launch([rs[1]], busy={id(a)})
    assert take == [] and rest == [rs[1]]


def test_pool_bytes_counts_slots_maps_and_handles():
    from crm_gb300.serving import pool_bytes
    cfg = S.config_64x58(nx=64)
    hb = lambda cap: 1000 * min(cap, 608)
    assert pool_bytes(cfg, 10, 3, hb) == 10 * slot_bytes(cfg) + 3 * 12 * 10 + 3 * 10000
    assert pool_bytes(cfg, 2048, 3, hb) - pool_bytes(cfg, 1024, 3, hb) == 1024 * (slot_bytes(cfg) + 36)
