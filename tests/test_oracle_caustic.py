"""The oracle's eye pass on the full caustic scene against the reference's own
hitpoints at step 51 (tests/golden/caustic_step51_row780.npz, made by
tests/golden/make_golden.py), including the NaN weight the reference gives
pixel 799031 there: its rough-dielectric BSDF value and pdf are NaN for the
direction sampled at the path's third glass interface, and the eye pass
(SPPM.cpp:278-281) goes on with them."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), 'oracle'))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), 'friendsrender-r-public_gb300'))
sys.path.insert(0, os.path.join(HERE, 'golden'))

FIXTURE = os.path.join(HERE, 'golden', 'caustic_step51_row780.npz')


def load_fixture():
    from frsppm import scenes
    import make_golden
    scene = scenes.caustic_box()
    fx = np.load(FIXTURE)
    assert str(fx['scene_sha']) == make_golden.scene_sha(scene)
    return scene, fx


def check_row(hp, fx, W):
    """hp: hitpoints of the whole frame as the oracle / library report them."""
    row = int(fx['row'])
    sl = slice(row * W, (row + 1) * W)
    np.testing.assert_array_equal(hp['type'][sl], fx['hp_type'])
    hit = fx['hp_type'] == 1
    np.testing.assert_array_equal(hp['facet'][sl][hit], fx['hp_facet'][hit])
    for k, f in (('pos', 'hp_pos'), ('nrm', 'hp_nrm'), ('out', 'hp_out'), ('rough', 'hp_rough')):
        np.testing.assert_array_equal(hp[k][sl][hit], fx[f][hit])
    # Weights: NaN in the same places, the rest within 1e-5 relative (the
    # tolerance of the other reference-parity tests: the product's rounding
    # order is not the reference's).
    w, wr = hp['w'][sl][hit].astype(np.float64), fx['hp_w'][hit].astype(np.float64)
    np.testing.assert_array_equal(np.isnan(w), np.isnan(wr))
    ok = ~np.isnan(wr)
    assert (np.abs(w[ok] - wr[ok]) <= 1e-5 * np.abs(wr[ok])).all()


def test_oracle_caustic_step51_matches_reference():
    import port_abi
    scene, fx = load_fixture()
    assert np.isnan(fx['hp_w'][799031 - 780 * 1024]).all()
    with port_abi.PortRenderer(scene, 1000, alpha=0.7, radius=0.01) as r:
        r.seek(int(fx['step']) - 1)
        r.iterate(1)
        check_row(r.read_hitpoints(), fx, scene['camera']['width'])
