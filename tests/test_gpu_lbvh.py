"""The device LBVH builder (FR_BVH_DEVICE_LBVH): a different tree, the same
hits.  Against the reference's golden hits and iterations, and against the
host SAH tree on the full mixed-materials scene."""
import time

import numpy as np
import pytest

from conftest import GOLDEN_SCENES, load_golden

pytestmark = pytest.mark.gpu

NAMES = sorted(GOLDEN_SCENES)


@pytest.mark.parametrize('name', NAMES)
def test_lbvh_hits_match_reference(name):
    from frsppm import abi
    gold = load_golden(name)
    with abi.Renderer(GOLDEN_SCENES[name](), int(gold['photons']), alpha=0.9, radius=0.015,
                      bvh_builder=abi.BVH_DEVICE_LBVH) as r:
        facet, tuv = r.trace_closest(gold['rays'])
        hit_any = r.trace_any(gold['any_rays'])
        np.testing.assert_array_equal(facet, gold['hit_facet'])
        hit = gold['hit_facet'] >= 0
        np.testing.assert_array_equal(tuv[hit], gold['hit_tuv'][hit])
        np.testing.assert_array_equal(hit_any, gold['any_hit'])
        for s in range(1, int(gold['iters']) + 1):
            r.iterate(1)
            hp = r.read_hitpoints()
            t = gold['it%d_hp_type' % s]
            np.testing.assert_array_equal(hp['type'] == 1, t == 1)
            np.testing.assert_array_equal(hp['pos'][t == 1], gold['it%d_hp_pos' % s][t == 1])
            _, path, slot = r.compacted_photons()
            np.testing.assert_array_equal(path, gold['it%d_ph_path' % s])
            np.testing.assert_array_equal(slot, gold['it%d_ph_slot' % s])
            np.testing.assert_array_equal(r.read_gather()[0], gold['it%d_gather_m' % s])


def test_lbvh_equals_sah_on_mixed_materials():
    from frsppm import abi, scenes
    scene = scenes.mixed_materials()
    rng = np.random.default_rng(7)
    lo, hi = scene['pos'].reshape(-1, 3).min(0), scene['pos'].reshape(-1, 3).max(0)
    n = 200_000
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([o, d, np.ones((n, 1))], 1).astype(np.float32)
    out = {}
    for b in (abi.BVH_HOST_SAH, abi.BVH_DEVICE_LBVH):
        t0 = time.perf_counter()
        with abi.Renderer(scene, 1000, alpha=0.7, radius=0.02, bvh_builder=b) as r:
            setup = time.perf_counter() - t0
            out[b] = r.trace_closest(rays) + (setup, r.stats()['bvh_nodes'])
    fa, ta, sa, na = out[abi.BVH_HOST_SAH]
    fb, tb, sb, nb = out[abi.BVH_DEVICE_LBVH]
    print('setup s: SAH %.2f LBVH %.2f; nodes %d / %d' % (sa, sb, na, nb))
    assert (fa >= 0).sum() > n // 4
    np.testing.assert_array_equal(fa, fb)
    np.testing.assert_array_equal(ta[fa >= 0], tb[fa >= 0])
