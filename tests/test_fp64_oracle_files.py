"""The committed FP64 CPU-converged oracle images (tests/golden/fp64_*.npz,
made by tests/golden/make_fp64_oracle.py) that bench.py and the GPU tests
measure renders against: each is finite and non-negative, covers its stated
window, and holds at least the photon paths its use assumes."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

CASES = {
    # name: (image shape, window, least photon paths)
    'caustic_crop': ((256, 256, 3), (384, 384, 640, 640), 2_000_000_000),
    'cornell': ((256, 256, 3), (0, 0, 0, 0), 400_000_000),
    'mixed_small': ((180, 320, 3), (0, 0, 0, 0), 150_000_000),
}


@pytest.mark.parametrize('name', sorted(CASES))
def test_fp64_oracle_file(name):
    shape, window, paths = CASES[name]
    d = np.load(os.path.join(GOLDEN, 'fp64_%s.npz' % name))
    L = d['radiance']
    assert L.shape == shape
    assert np.isfinite(L).all() and (L >= 0).all() and L.mean() > 0
    assert tuple(int(v) for v in d['window']) == window
    assert int(d['photon_paths']) == int(d['iterations']) * int(d['photons_per_iteration'])
    assert int(d['photon_paths']) >= paths
    assert int(d['stream_key']) == 0x4F524331  # streams of its own
