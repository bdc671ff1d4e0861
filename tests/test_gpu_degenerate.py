"""FR_FLAG_END_DEGENERATE_PATHS on the full caustic scene, where the
reference's eye pass at step 51 gives pixel 799031 a NaN weight (its
rough-dielectric BSDF value and pdf are NaN for one sampled direction).

* Without the flag the library's hitpoints of that step equal the reference's
  own (tests/golden/caustic_step51_row780.npz), NaN included.
* With it that path ends without a hitpoint and nothing else changes."""
import numpy as np
import pytest

from test_oracle_caustic import check_row, load_fixture

pytestmark = pytest.mark.gpu


def _step_hitpoints(scene, step, flags):
    from frsppm import abi
    with abi.Renderer(scene, 1000, alpha=0.7, radius=0.01, flags=flags) as r:
        r.seek(step - 1)
        r.iterate(1)
        return r.read_hitpoints()


def test_caustic_step51_matches_reference():
    scene, fx = load_fixture()
    hp = _step_hitpoints(scene, int(fx['step']), 0)
    check_row(hp, fx, scene['camera']['width'])
    assert np.isnan(hp['w'][799031]).all()


def test_end_degenerate_paths_flag():
    from frsppm import abi
    scene, fx = load_fixture()
    plain = _step_hitpoints(scene, int(fx['step']), 0)
    ended = _step_hitpoints(scene, int(fx['step']), abi.FLAG_END_DEGENERATE_PATHS)
    assert plain['type'][799031] == 1 and ended['type'][799031] != 1
    other = np.ones(len(plain['type']), bool)
    other[799031] = False
    np.testing.assert_array_equal(plain['type'][other], ended['type'][other])
    hit = other & (plain['type'] == 1)
    for k in ('pos', 'w', 'facet'):
        np.testing.assert_array_equal(plain[k][hit], ended[k][hit])
    assert np.isfinite(ended['w'][ended['type'] == 1]).all()


def test_guided_caustic_stays_finite():
    """Guided photons bounce long inside the cluster of rough-dielectric
    spheres; a path's flux and PDF products then overflow together and its
    photons carry inf / inf.  With the flag such a path ends, and the guided
    render of the full caustic scene stays finite (without it, pixels turned
    NaN after about 22 iterations)."""
    from frsppm import abi, scenes
    scene = scenes.caustic_box()
    flags = abi.FLAG_STANDARD_RESOLVE | abi.FLAG_END_DEGENERATE_PATHS
    with abi.Renderer(scene, 2_000_000, alpha=0.7, radius=0.01, guide=True, flags=flags) as r:
        for _ in range(8):
            r.iterate(5)
            img = r.resolve()
            assert np.isfinite(img).all(), r.read_state()['n'].sum()
        pos, flux, d, counts = r.read_photon_slots()
        live = d[:, 3] != 0
        assert np.isfinite(flux[live]).all()
