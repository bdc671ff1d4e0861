"""CPU restatement of the reference's image output, for tests only (the
oracle; the library's own path is the k_export_rgba8 kernel).

ExportPNG (SPPM/SPPM/TextureUtility.cpp:52-65) writes pixel (i, j) as the
render target sampled by LinearSampler::Sample (TextureSampler.h:61-79) at
u = i / W, v = j / H, each channel max(0, min(255, int(c * 255))).  Pinned to
the reference's own PNG of the golden fixtures' images (tests/test_png.py).
"""
import numpy as np


def export_rgba8(image, width, height):
    """image: (height*width, 4) float32 RGBA, row-major; returns (height,
    width, 4) uint8.  All arithmetic in float32 in the reference's order."""
    f = np.float32
    im = np.asarray(image, np.float32).reshape(height, width, 4)
    u = (np.arange(width, dtype=f) / f(width)).astype(f)
    v = (np.arange(height, dtype=f) / f(height)).astype(f)
    iu = (f(width) * u).astype(np.int32)
    iv = (f(height) * v).astype(np.int32)
    x1, y1 = np.abs(iu) % width, np.abs(iv) % height
    x2, y2 = np.minimum(width - 1, x1 + 1), np.minimum(height - 1, y1 + 1)
    w = (np.abs(u * f(width)) - np.abs(iu).astype(f)).astype(f)[None, :, None]
    h = (np.abs(v * f(height)) - np.abs(iv).astype(f)).astype(f)[:, None, None]
    t00, t10 = im[y1][:, x1], im[y1][:, x2]
    t01, t11 = im[y2][:, x1], im[y2][:, x2]
    up = (t00 * (f(1) - w) + t10 * w).astype(f)
    down = (t01 * (f(1) - w) + t11 * w).astype(f)
    c = (up * (f(1) - h) + down * h).astype(f)
    s = (c * f(255)).astype(np.float64)
    # int(x) of the reference's x86 build: truncation, INT_MIN for NaN and
    # out-of-range values (0 after the clamp).
    bad = ~np.isfinite(s) | (np.abs(s) >= 2.0 ** 31)
    q = np.where(bad, -2 ** 31, np.trunc(np.where(bad, 0, s))).astype(np.int64)
    return np.clip(q, 0, 255).astype(np.uint8)
