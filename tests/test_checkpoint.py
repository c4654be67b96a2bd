"""Restart files: the pbuf 'global' CRM fields round-trip exactly, and a
GCM step resumed from a checkpoint equals an uninterrupted run (oracle)."""
import numpy as np
import pytest

import oracle
from crm_gb300 import checkpoint as CK
from crm_gb300 import crm_types as T
from crm_gb300 import synthetic as S


def test_round_trip(tmp_path):
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=3, moist=True)
    p = str(tmp_path / 'crm.ckpt')
    CK.save(p, cfg, st, rad.qrad, list(desc._keep))
    cfg2, st2, qrad2, gcol2 = CK.load(p)
    assert cfg2 == cfg
    assert gcol2 == [int(g) for g in desc._keep]
    for n, a in st.arrays().items():
        b = getattr(st2, n)
        assert b.flags.f_contiguous and np.array_equal(a, b), n
    assert np.array_equal(qrad2, rad.qrad)
    with open(p, 'rb') as f:
        assert f.read(9) == CK.MAGIC


def test_rejects_foreign_and_truncated(tmp_path):
    p = tmp_path / 'bad'
    p.write_bytes(b'not a checkpoint')
    with pytest.raises(ValueError):
        CK.load(str(p))
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=2)
    q = str(tmp_path / 'ok')
    CK.save(q, cfg, st, rad.qrad, list(desc._keep))
    data = open(q, 'rb').read()
    open(q, 'wb').write(data[:-100])
    with pytest.raises(ValueError):
        CK.load(q)


def test_resume_equals_uninterrupted(tmp_path):
    """Two GCM steps in a row == one step, checkpoint, restart, second step."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=3, moist=True)
    desc.dt_gl = 400.0
    a_st, a_rad = st.copy(), rad.copy()
    for igstep in (1, 2):
        desc.igstep = igstep
        assert oracle.run(cfg, desc, cin, a_st, a_rad)[0] == 0
    b_st, b_rad = st.copy(), rad.copy()
    desc.igstep = 1
    assert oracle.run(cfg, desc, cin, b_st, b_rad)[0] == 0
    p = str(tmp_path / 'step1.ckpt')
    CK.save(p, cfg, b_st, b_rad.qrad, list(desc._keep))
    cfg2, st2, qrad2, gcol2 = CK.load(p)
    rad2 = T.CrmRad.zeros(3, cfg2.crm_nx_rad, 1, cfg2.crm_nz)
    rad2.qrad[...] = qrad2
    d2 = T.call_desc(3, 3, 400.0, 2, gcol2)
    assert oracle.run(cfg2, d2, cin, st2, rad2)[0] == 0
    for n, v in a_st.arrays().items():
        assert np.array_equal(v, getattr(st2, n)), n
