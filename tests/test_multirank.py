"""The N > 1 host path on CPU: columns sharded over 2 gloo ranks, each rank
integrating its own block with the oracle, results gathered on rank 0 and
compared bit for bit with one process integrating all columns.  This is the
partitioning bench.py uses with one rank per GPU (no collective on the data
path; a barrier and a max-over-ranks of the timings)."""
import os
import socket

import numpy as np
import pytest

from crm_gb300.shard import column_shard, shard_bounds

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NCOLS = 5


def test_column_shard_partitions():
    for n in (1, 5, 1024, 1027):
        for w in (1, 2, 3, 8):
            b = shard_bounds(n, w)
            assert sum(c for _, c in b) == n
            assert b[0][0] == 0
            for (f0, c0), (f1, _) in zip(b, b[1:]):
                assert f0 + c0 == f1
            assert max(c for _, c in b) - min(c for _, c in b) <= 1
    with pytest.raises(ValueError):
        column_shard(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, outdir):
    import sys
    for p in (os.path.join(REPO, 'acme-ecp_gb300'), os.path.join(REPO, 'oracle')):
        sys.path.insert(0, p)
    import torch.distributed as dist
    import oracle
    from crm_gb300 import crm_types as T
    from crm_gb300 import synthetic as S
    from crm_gb300.shard import column_shard, gather_columns
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=NCOLS, moist=True)
    first, count = column_shard(NCOLS, rank, world)
    cols = list(range(first, first + count))
    d = T.call_desc(count, count, 200.0, desc.igstep, np.asarray(desc._keep)[cols])
    st_l, rad_l = st.take(cols), rad.take(cols)
    rc, stat, out = oracle.run(cfg, d, cin.take(cols), st_l, rad_l, nthreads=2)
    assert rc == 0
    res = {}
    for n, a in st_l.arrays().items():
        res['state.' + n] = gather_columns(np.ascontiguousarray(a), NCOLS, world, dist.all_gather)
    for n in ('precc', 'cltot', 'sltend', 'qltend'):
        res['out.' + n] = gather_columns(np.ascontiguousarray(getattr(out, n)), NCOLS, world,
                                         dist.all_gather)
    dist.barrier()
    if rank == 0:
        np.savez(os.path.join(outdir, 'gathered.npz'), **res)
    dist.destroy_process_group()


def test_two_gloo_ranks_match_one_process(tmp_path):
    import torch.multiprocessing as mp
    import oracle
    from crm_gb300 import synthetic as S
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    got = np.load(os.path.join(tmp_path, 'gathered.npz'))
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=NCOLS, moist=True)
    desc.dt_gl = 200.0
    rc, stat, out = oracle.run(cfg, desc, cin, st, rad)
    assert rc == 0
    for n, a in st.arrays().items():
        assert np.array_equal(got['state.' + n], a), n
    for n in ('precc', 'cltot', 'sltend', 'qltend'):
        assert np.array_equal(got['out.' + n], getattr(out, n)), n
