"""Sharded SPPM iteration on CPU ranks (gloo, world size 2): each rank gathers
only the photons of its own path range; the all-reduced counts equal the
reference's per-hitpoint photon counts (golden fixtures) exactly, and the
N/R/NumGather update applied to them on every rank reproduces the
reference's state."""
import os
import socket

import numpy as np
import pytest

from conftest import GOLDEN, load_golden


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _update(n, r, g, m, alpha):
    """applyHitPointInfo's update of N, R and NumGather (SPPM.cpp:444-449) in
    the reference's float32 arithmetic."""
    n, r, g = n.copy(), r.copy(), g.copy()
    hit = m > 0
    a = n[hit].astype(np.float32) + np.float32(alpha) * m[hit].astype(np.float32)
    b = (n[hit] + m[hit]).astype(np.float32)
    r[hit] = r[hit] * np.sqrt(a / b, dtype=np.float32)
    n[hit] = (n[hit].astype(np.float32) + m[hit].astype(np.float32) * np.float32(alpha)).astype(np.int32)
    g[hit] += 1
    return n, r, g


def _rank_main(rank, world, port, name, out):
    import sys
    import torch.distributed as dist
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path[:0] = [here, os.path.join(os.path.dirname(here), 'oracle'),
                    os.path.join(os.path.dirname(here), 'friendsrender-r-public_gb300')]
    import port_abi
    from frsppm import shard
    dist.init_process_group('gloo', init_method='tcp://127.0.0.1:%d' % port, rank=rank, world_size=world)
    try:
        gold = dict(np.load(os.path.join(GOLDEN, name + '.npz')))
        paths = int(gold['photons'])
        lo, hi = shard.path_range(rank, world, paths)
        n = np.zeros(len(gold['it1_sp_n']), np.int32)
        r = np.full(len(n), np.float32(0.015), np.float32)
        g = np.zeros(len(n), np.int32)
        for s in range(1, int(gold['iters']) + 1):
            hit = gold['it%d_hp_type' % s] == 1
            mine = (gold['it%d_ph_path' % s] >= lo) & (gold['it%d_ph_path' % s] < hi)
            ph = gold['it%d_ph' % s][mine]
            m = np.zeros(len(n), np.int32)
            m[hit] = port_abi.radius_count(gold['it%d_hp_pos' % s][hit], r[hit], ph[:, :3])
            phi = np.zeros((len(n), 3), np.float32)
            m_all, _ = shard.reduce_partials(m, phi)
            np.testing.assert_array_equal(m_all, gold['it%d_gather_m' % s])
            n, r, g = _update(n, r, g, m_all, 0.9)
            np.testing.assert_array_equal(n, gold['it%d_sp_n' % s])
            np.testing.assert_array_equal(r, gold['it%d_sp_r' % s])
            np.testing.assert_array_equal(g, gold['it%d_sp_g' % s])
        out.put((rank, 'ok'))
    except Exception as e:  # reported to the parent
        out.put((rank, repr(e)))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize('name', ['cornell32', 'mixed48x32'])
def test_sharded_counts_and_update_match_reference(name):
    import multiprocessing as mp
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(k, 2, port, name, q)) for k in range(2)]
    for p in procs:
        p.start()
    results = dict(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert results == {0: 'ok', 1: 'ok'}, results


def test_path_ranges_partition():
    from frsppm import shard
    for world in (1, 2, 3, 8):
        for paths in (0, 1, 7, 1000, 1000003):
            ranges = [shard.path_range(k, world, paths) for k in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == paths
            assert all(ranges[k][1] == ranges[k + 1][0] for k in range(world - 1))
            assert max(h - l for l, h in ranges) - min(h - l for l, h in ranges) <= 1
