"""fr_iterate_batch and fr_autotune: a batch of uneven scenes advanced
together gives each scene exactly what fr_iterate gives it alone, and the
autotuner's iterations are ordinary iterations (its threshold changes the
speed only)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scenes():
    from frsppm import scenes
    return [(scenes.cornell_box(width=32, height=32), 3000), (scenes.small_mixed(), 5000),
            (scenes.small_caustic(), 20000)]


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


def test_batch_equals_single():
    from frsppm import abi
    pairs = [(abi.Renderer(sc, p, alpha=0.7, radius=0.02), abi.Renderer(sc, p, alpha=0.7, radius=0.02))
             for sc, p in _scenes()]
    try:
        abi.iterate_batch([a for a, _ in pairs], 3)
        for _, b in pairs:
            b.iterate(3)
        for a, b in pairs:
            _same(a, b)
    finally:
        for a, b in pairs:
            a.close()
            b.close()


def test_autotune_iterations_are_ordinary():
    from frsppm import abi
    sc, p = _scenes()[2]
    with abi.Renderer(sc, p, alpha=0.7, radius=0.02) as a, abi.Renderer(sc, p, alpha=0.7, radius=0.02) as b:
        t = a.autotune(1)
        assert t in (4096, 8192, 16384, 32768, 65536)
        b.iterate(10)  # fr_autotune ran 5 x (1 + 1) iterations
        _same(a, b)
        a.iterate(2)
        b.iterate(2)
        _same(a, b)


def test_batch_graph_equals_single():
    """fr_batch_create / fr_batch_iterate: one graph launch per iteration for
    all the scenes gives each scene what fr_iterate gives it, also when
    batch iterations and a context's own iterations alternate."""
    from frsppm import abi
    pairs = [(abi.Renderer(sc, p, alpha=0.7, radius=0.02), abi.Renderer(sc, p, alpha=0.7, radius=0.02))
             for sc, p in _scenes()]
    try:
        with abi.Batch([a for a, _ in pairs]) as batch:
            batch.iterate(2)
            pairs[1][0].iterate(1)
            batch.iterate(1)
        for j, (_, b) in enumerate(pairs):
            b.iterate(4 if j == 1 else 3)
        for a, b in pairs:
            _same(a, b)
            np.testing.assert_array_equal(a.resolve(), a.resolve())
        assert pairs[0][0].stats()['iterations'] == 3
    finally:
        for a, b in pairs:
            a.close()
            b.close()
