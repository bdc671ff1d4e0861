"""An iteration's gather runs on the pixel stream beside the next iteration's
photon pass, and fr_resolve_async resolves on the pixel stream.  A context
iterated back to back must hold what a context synchronized after every
iteration holds (nothing overlaps there): hitpoints, photon sets, N, R and
NumGather bit for bit, and the images read back on the way must be the
images of the iterations they were asked after."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scenes():
    from frsppm import scenes
    return [(scenes.small_mixed(), 5000, {}), (scenes.small_caustic(), 20000, {}),
            (scenes.small_caustic(), 20000, {'guide': True, 'guide_seed': 3})]


def _same(a, b):
    ha, hb = a.read_hitpoints(), b.read_hitpoints()
    np.testing.assert_array_equal(ha['type'], hb['type'])
    np.testing.assert_array_equal(ha['pos'], hb['pos'])
    pa, path_a, slot_a = a.compacted_photons()
    pb, path_b, slot_b = b.compacted_photons()
    np.testing.assert_array_equal(path_a, path_b)
    np.testing.assert_array_equal(slot_a, slot_b)
    np.testing.assert_array_equal(pa[:, :3], pb[:, :3])
    sa, sb = a.read_state(), b.read_state()
    np.testing.assert_array_equal(sa['n'], sb['n'])
    np.testing.assert_array_equal(sa['r'], sb['r'])
    np.testing.assert_array_equal(sa['g'], sb['g'])
    # Flux sums can differ in the last bits between runs (atomic order).
    assert np.abs(sa['tau'] - sb['tau']).max() <= 1e-6 * max(1e-30, np.abs(sb['tau']).max())


@pytest.mark.parametrize('case', range(3))
def test_back_to_back_equals_synchronized(case):
    from frsppm import abi
    scene, photons, extra = _scenes()[case]
    kw = dict(alpha=0.7, radius=0.02, flags=abi.FLAG_END_DEGENERATE_PATHS, **extra)
    with abi.Renderer(scene, photons, **kw) as a, abi.Renderer(scene, photons, **kw) as b:
        a.iterate(7, sync=False)
        a.synchronize()
        for _ in range(7):
            b.iterate(1)  # synchronizes
        _same(a, b)


def test_async_images_follow_their_iterations():
    """Images queued by fr_resolve_async between back-to-back iterations equal
    fr_resolve of a synchronized twin after the same number of iterations
    (up to the last bits of the flux sums)."""
    import torch
    from frsppm import abi, scenes
    scene = scenes.small_mixed()
    kw = dict(alpha=0.7, radius=0.02)
    with abi.Renderer(scene, 5000, **kw) as a, abi.Renderer(scene, 5000, **kw) as b:
        n = a.width * a.height
        hosts = [torch.empty((n, 4), dtype=torch.float32, pin_memory=True) for _ in range(4)]
        tickets = []
        for k in range(4):
            a.iterate(1, sync=False)
            tickets.append(a.resolve_async(hosts[k].data_ptr()))
            if k >= 1:
                a.resolve_wait(tickets[k - 1])
        a.resolve_wait(tickets[-1])
        a.synchronize()
        # Two device images are used in turn, so each image is checked once
        # its own copy has landed and before a later call reuses the buffer:
        # the host buffers are distinct, so all four stay readable.
        for k in range(4):
            b.iterate(1)
            ref = b.resolve()
            got = hosts[k].numpy()
            scale = max(1e-30, float(np.abs(ref).max()))
            assert np.abs(got - ref).max() <= 1e-5 * scale, k
