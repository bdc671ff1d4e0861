"""GPU path against the reference's own CPU code (golden fixtures made by
tests/golden/make_golden.py from the reference built with the Philox overlay).

Bit-exact: closest-hit facet ids and t/u/v, any-hit bits, hitpoint types and
facets, the compacted photon set (path, slot), per-hitpoint photon counts M,
N and NumGather.  Within 1e-4 relative (FP32 summation order, FP64 tau on the
GPU against FP32 in the reference): flux sums, tau, the image.
"""
import numpy as np
import pytest

from conftest import GOLDEN_SCENES, load_golden

pytestmark = pytest.mark.gpu

NAMES = sorted(GOLDEN_SCENES)


def _renderer(name, gold, **kw):
    from frsppm import abi
    return abi.Renderer(GOLDEN_SCENES[name](), int(gold['photons']), alpha=0.9, radius=0.015, **kw)


def _rel(a, b, floor):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


@pytest.mark.parametrize('name', NAMES)
def test_closest_hit_matches_reference(name):
    gold = load_golden(name)
    with _renderer(name, gold) as r:
        facet, tuv = r.trace_closest(gold['rays'])
    ref_f = gold['hit_facet']
    assert (ref_f >= 0).sum() > len(ref_f) // 4
    np.testing.assert_array_equal(facet, ref_f)
    hit = ref_f >= 0
    np.testing.assert_array_equal(tuv[hit], gold['hit_tuv'][hit])


@pytest.mark.parametrize('name', NAMES)
def test_any_hit_matches_reference(name):
    gold = load_golden(name)
    with _renderer(name, gold) as r:
        hit = r.trace_any(gold['any_rays'])
    np.testing.assert_array_equal(hit, gold['any_hit'])


@pytest.mark.parametrize('name', NAMES)
def test_iterations_match_reference(name):
    gold = load_golden(name)
    iters = int(gold['iters'])
    with _renderer(name, gold) as r:
        for s in range(1, iters + 1):
            r.iterate(1)
            hp = r.read_hitpoints()
            t_ref = gold['it%d_hp_type' % s]
            # NONE and ONLY_DIRECTLIGHT both skip the gather (SPPM.cpp:409-422).
            np.testing.assert_array_equal(hp['type'] == 1, t_ref == 1, err_msg='hitpoint types, iteration %d' % s)
            hit = t_ref == 1
            np.testing.assert_array_equal(hp['facet'][hit], gold['it%d_hp_facet' % s][hit])
            np.testing.assert_array_equal(hp['pos'][hit], gold['it%d_hp_pos' % s][hit])
            np.testing.assert_array_equal(hp['nrm'][hit], gold['it%d_hp_nrm' % s][hit])
            np.testing.assert_array_equal(hp['out'][hit], gold['it%d_hp_out' % s][hit])
            np.testing.assert_array_equal(hp['rough'][hit], gold['it%d_hp_rough' % s][hit])
            assert _rel(hp['w'][hit], gold['it%d_hp_w' % s][hit], 1e-30).max() < 1e-5

            ph, path, slot = r.compacted_photons()
            np.testing.assert_array_equal(path, gold['it%d_ph_path' % s])
            np.testing.assert_array_equal(slot, gold['it%d_ph_slot' % s])
            ref_ph = gold['it%d_ph' % s]
            np.testing.assert_array_equal(ph[:, 0:3], ref_ph[:, 0:3])   # positions
            np.testing.assert_array_equal(ph[:, 6:10], ref_ph[:, 6:10])  # incoming direction, index
            assert _rel(ph[:, 3:6], ref_ph[:, 3:6], 1e-30).max() < 1e-4  # flux
            assert _rel(ph[:, 10], ref_ph[:, 10], 1e-30).max() < 1e-4    # pdf

            m, phi = r.read_gather()
            np.testing.assert_array_equal(m, gold['it%d_gather_m' % s])
            ref_phi = gold['it%d_gather_phi' % s]
            scale = np.abs(ref_phi).max()
            assert np.abs(phi - ref_phi).max() <= 1e-4 * scale + 1e-30

            st = r.read_state()
            np.testing.assert_array_equal(st['n'], gold['it%d_sp_n' % s])
            np.testing.assert_array_equal(st['g'], gold['it%d_sp_g' % s])
            np.testing.assert_array_equal(st['r'], gold['it%d_sp_r' % s])
            ref_tau = gold['it%d_sp_rad' % s]
            assert np.abs(st['tau'] - ref_tau).max() <= 1e-4 * np.abs(ref_tau).max() + 1e-30
            if 'it%d_hp_dl' % s in gold:  # environment light (IBL)
                # HIT / ONLY_DIRECTLIGHT / NONE as the reference's.
                np.testing.assert_array_equal(hp['type'], t_ref)
                last, tot, cnt = r.read_direct()
                np.testing.assert_array_equal(cnt, gold['it%d_sp_ndl' % s])
                for got, ref in ((last, gold['it%d_hp_dl' % s]), (tot, gold['it%d_sp_dl' % s])):
                    assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max() + 1e-30
        img = r.resolve()
    ref = gold['image']
    assert np.isfinite(img).all()
    # Per pixel and channel: within 1e-4 of the reference's own value, with
    # an absolute floor of 1e-7 of the image maximum for pixels near zero.
    a, b = img[:, :3].astype(np.float64), ref[:, :3].astype(np.float64)
    bad = np.abs(a - b) > 1e-4 * np.abs(b) + 1e-7 * np.abs(b).max()
    assert not bad.any(), (int(bad.sum()), _rel(img[:, :3][bad], ref[:, :3][bad], 1e-30).max())
