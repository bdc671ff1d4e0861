"""Photon radius query on the GPU grid against an exhaustive float32
evaluation of the reference's predicate: isIncludePoint(p, x - R, x + R)
(kdtree.h:78-88) and |p - x|^2 < R^2 (SPPM.cpp:432), bit-exact per pair."""
import numpy as np
import pytest

from conftest import GOLDEN_SCENES

pytestmark = pytest.mark.gpu


def brute_pairs(hp, R, ph):
    f32 = np.float32
    hp = hp.astype(f32)
    R = R.astype(f32)
    ph = ph.astype(f32)
    bmin = hp - R[:, None] * f32(1)
    bmax = hp + R[:, None] * f32(1)
    R2 = R * R
    out = []
    for i in range(len(hp)):
        inside = np.all((bmin[i] <= ph) & (bmax[i] >= ph), axis=1)
        d = ph - hp[i]
        n2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        j = np.nonzero(inside & (n2 < R2[i]))[0]
        out.append(j)
    return out


def _case(seed, nh, np_, surface):
    rng = np.random.Generator(np.random.PCG64(seed))
    if surface:
        # Photons and hitpoints on a few planes (the distribution SPPM produces).
        ph = rng.uniform(0, 1, (np_, 3)).astype(np.float32)
        ph[:, 1] = rng.choice([0.0, 0.5, 1.0], np_)
        hp = rng.uniform(0, 1, (nh, 3)).astype(np.float32)
        hp[:, 1] = rng.choice([0.0, 0.5, 1.0], nh)
    else:
        ph = rng.uniform(-1, 1, (np_, 3)).astype(np.float32)
        hp = rng.uniform(-1, 1, (nh, 3)).astype(np.float32)
    R = rng.uniform(0.005, 0.06, nh).astype(np.float32)
    return hp, R, ph


@pytest.mark.parametrize('seed,surface', [(1, True), (2, False), (3, True)])
@pytest.mark.parametrize('cell', [0.02, 0.05, 0.2])
def test_radius_query_pairs_exact(seed, surface, cell):
    from frsppm import abi
    hp, R, ph = _case(seed, 1500, 20000, surface)
    with abi.Renderer(GOLDEN_SCENES['cornell32'](), 64) as r:
        counts, pairs = r.radius_query(hp, R, ph, cell, pairs_capacity=2_000_000)
    ref = brute_pairs(hp, R, ph)
    np.testing.assert_array_equal(counts, [len(j) for j in ref])
    got = {(int(a), int(b)) for a, b in pairs}
    want = {(i, int(j)) for i, js in enumerate(ref) for j in js}
    assert len(pairs) == len(got)  # no pair reported twice
    assert got == want


def test_radius_query_empty_inputs():
    from frsppm import abi
    with abi.Renderer(GOLDEN_SCENES['cornell32'](), 64) as r:
        counts, _ = r.radius_query(np.zeros((5, 3)), np.full(5, 0.1), np.zeros((0, 3)), 0.1)
        assert (counts == 0).all()
        counts, _ = r.radius_query(np.zeros((0, 3)), np.zeros(0), np.zeros((3, 3)), 0.1)
        assert counts.shape == (0,)


def test_radius_query_refuses_unbounded_balls():
    """A radius that is not finite or negative, or a ball more than 128 cells
    wide, is refused with FR_ERR_INVALID before any kernel runs; the context
    stays usable."""
    from frsppm import abi
    ph = np.random.Generator(np.random.PCG64(5)).uniform(0, 1, (1000, 3)).astype(np.float32)
    hp = np.full((3, 3), 0.5, np.float32)
    with abi.Renderer(GOLDEN_SCENES['cornell32'](), 64) as r:
        for bad in (np.nan, np.inf, -0.01, 3.0):
            R = np.array([0.05, bad, 0.05], np.float32)
            with pytest.raises(RuntimeError, match='radius'):
                r.radius_query(hp, R, ph, 0.02)
        counts, _ = r.radius_query(hp, np.full(3, 0.05, np.float32), ph, 0.02)
        assert (counts == [len(j) for j in brute_pairs(hp, np.full(3, 0.05, np.float32), ph)]).all()
