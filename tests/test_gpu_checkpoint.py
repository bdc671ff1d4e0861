"""fr_save_state / fr_load_state: a render interrupted after k iterations and
resumed in a fresh context continues exactly as the uninterrupted render
(hitpoints, photon slots, N, R, NumGather bit for bit; tau and the image to
the last bits of the FP32 flux sums, whose photon order within a grid cell
follows the GPU's atomic ranks).  Mismatched contexts are refused."""
import numpy as np
import pytest

from frsppm import abi

pytestmark = pytest.mark.gpu


def _scene():
    from frsppm import scenes
    return scenes.mixed_materials(width=96, height=64, n_spheres=16, field_n=32, tex_size=64, light_tex=32,
                                  n_lat=10, n_lon=12, extent=0.8, aperture=0.05)


def _snapshot(r):
    st = r.read_state()
    pos, flux, d, counts = r.read_photon_slots()
    return st, r.read_hitpoints(), (pos, flux, d, counts), r.resolve()


def _check_same(a, b):
    sa, ha, pa, ia = a
    sb, hb, pb, ib = b
    for k in ('n', 'r', 'g'):
        np.testing.assert_array_equal(sa[k], sb[k])
    np.testing.assert_allclose(sa['tau'], sb['tau'], rtol=1e-6, atol=1e-6 * np.abs(sa['tau']).max())
    np.testing.assert_array_equal(ha['type'], hb['type'])
    hit = ha['type'] == 1   # records of pixels without a hitpoint are not state
    for k in ('pos', 'nrm', 'out', 'facet', 'rough', 'w', 'mat'):
        np.testing.assert_array_equal(ha[k][hit], hb[k][hit])
    for x, y in zip(pa, pb):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_allclose(ia, ib, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize('flags,guide', [(0, False), (1, False), (abi.FLAG_END_DEGENERATE_PATHS, True)])
def test_resume_matches_uninterrupted(flags, guide):
    """Guided: the checkpoint also holds the network, its optimizer state and
    the copy the next emission samples (the training's weights one iteration
    behind), so the resumed render trains the same network bit for bit."""
    scene = _scene()
    kw = dict(alpha=0.7, radius=0.02, flags=flags, guide=guide, guide_seed=5)
    with abi.Renderer(scene, 15000, **kw) as a:
        a.iterate(3)
        ckpt = a.save_state()
        a.iterate(2)
        want = _snapshot(a)
        stats_a = a.stats()
        params_a = a.guide_params() if guide else None
    with abi.Renderer(scene, 15000, **kw) as b:
        b.iterate(1)                       # state to be overwritten
        b.load_state(ckpt)
        b.iterate(2)
        got = _snapshot(b)
        stats_b = b.stats()
        params_b = b.guide_params() if guide else None
    assert stats_a['iterations'] == stats_b['iterations'] == 5
    assert stats_a['photon_paths'] == stats_b['photon_paths']
    _check_same(want, got)
    if guide:
        np.testing.assert_array_equal(params_a, params_b)


def test_checkpoint_size_and_refusals():
    scene = _scene()
    with abi.Renderer(scene, 15000, alpha=0.7, radius=0.02) as a:
        a.iterate(1)
        ckpt = a.save_state()
        npix, slots = 96 * 64, 15000 * 32
        assert len(ckpt) == 56 + npix * (24 + 4 + 4 + 4 + 16) + slots * 48
        a.load_state(ckpt)                 # same context: accepted
        with pytest.raises(RuntimeError):
            a.load_state(ckpt[:-1])        # truncated
        bad = bytearray(ckpt)
        bad[0:8] = b'NOTSPPM!'
        with pytest.raises(RuntimeError):
            a.load_state(bytes(bad))
    with abi.Renderer(scene, 16000, alpha=0.7, radius=0.02) as other:
        with pytest.raises(RuntimeError):
            other.load_state(ckpt)         # another photon count
    with abi.Renderer(scene, 15000, alpha=0.8, radius=0.02) as other:
        with pytest.raises(RuntimeError):
            other.load_state(ckpt)         # another alpha
