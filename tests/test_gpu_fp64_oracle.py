"""Plain GPU renders against the FP64 CPU-converged oracle images
(tests/golden/fp64_*.npz, made by tests/golden/make_fp64_oracle.py): the
renderer's estimate converges to the oracle's.  The Cornell box (256^2, 100k
photon paths per iteration, alpha 0.7, r0 0.02; the oracle holds 4096
iterations): relMSE falls as iterations accumulate, is below 1% after 256
iterations, and the image's mean radiance is within 1% of the oracle's.
Renders are deterministic up to the last bits of the flux sums, so these
figures repeat run to run."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _oracle(name):
    d = np.load(os.path.join(GOLDEN, 'fp64_%s.npz' % name))
    return d['radiance'].astype(np.float64), int(d['iterations'])


def _rel_mse(img, width, ref):
    a = img[:, :3].astype(np.float64).reshape(-1, width, 3) ** 1.2   # resolve's gamma undone
    k = 1.0 / ref.mean()
    a, b = a * k, ref * k
    return float(((a - b) ** 2 / (b * b + 1e-2)).mean()), float(a.mean())


def test_cornell_converges_to_fp64_oracle():
    from frsppm import abi, scenes
    ref, iters = _oracle('cornell')
    assert iters >= 1024
    scene = scenes.cornell_box()
    errs = []
    with abi.Renderer(scene, 100_000, alpha=0.7, radius=0.02, flags=abi.FLAG_STANDARD_RESOLVE) as r:
        done = 0
        for m in (16, 64, 256):
            r.iterate(m - done)
            done = m
            e, mean = _rel_mse(r.resolve(), scene['camera']['width'], ref)
            errs.append(e)
    print('relMSE at 16 / 64 / 256 iterations: %.5f / %.5f / %.5f, mean radiance %.4f of the oracle\'s'
          % (errs[0], errs[1], errs[2], mean))
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 1e-2
    assert abs(mean - 1.0) < 1e-2
