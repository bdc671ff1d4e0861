"""bench.py's host-side helpers, on the CPU: the trace kernel's DRAM traffic
read from the committed ncu summary (the roofline line's `traffic`), the
relMSE against the FP64 oracle images, and the scene-size arithmetic the
timed line's L2 statement quotes."""
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402


def test_trace_traffic_from_committed_profile():
    t = bench.trace_traffic_per_launch()
    assert t is not None
    # Above the algorithmic bytes of a launch that traced rays (about 3.0 M rays
    # of 52 B over 13 launches, 12 MB), below a whole iteration's trace traffic.
    algorithmic = 3.0e6 * bench.TRACE_BYTES_PER_RAY / 13
    assert algorithmic < t < 700e6


def _resolved(radiance):
    """Pixels as fr_resolve writes them: radiance^(1/1.2), alpha 1."""
    img = np.ones((radiance.shape[0] * radiance.shape[1], 4), np.float32)
    img[:, :3] = (radiance.reshape(-1, 3) ** (1 / 1.2)).astype(np.float32)
    return img


def test_rel_mse_linear_properties():
    rng = np.random.default_rng(3)
    ref = rng.uniform(0.1, 2.0, (8, 12, 3))
    width = 12
    # The image of the reference itself: zero (up to the float32 round trip).
    assert bench.rel_mse_linear(_resolved(ref), width, ref, (0, 0, 0, 0)) < 1e-10
    # Scale-free: the same relative error on a 1000x brighter scene.
    noisy = ref * rng.uniform(0.8, 1.2, ref.shape)
    e1 = bench.rel_mse_linear(_resolved(noisy), width, ref, (0, 0, 0, 0))
    e2 = bench.rel_mse_linear(_resolved(noisy * 1000.0), width, ref * 1000.0, (0, 0, 0, 0))
    assert e1 > 0 and abs(e1 - e2) <= 1e-5 * e1
    # A window: the image is cropped to it before the comparison.
    full = rng.uniform(0.1, 2.0, (16, 20, 3))
    window = (4, 2, 16, 10)
    crop = full[2:10, 4:16]
    assert bench.rel_mse_linear(_resolved(full), 20, crop, window) < 1e-10


def test_scene_bytes():
    stats = {'bvh_nodes': 192053, 'triangles': 997444}
    b = bench.scene_bytes(stats)
    assert b == 192053 * 224 + 997444 * (48 + 64) + 3 * 1024 * 1024 * 4 + 512 * 512 * 4
    assert b > 129e6  # the mixed-materials scene alone is larger than the 129 MB L2
