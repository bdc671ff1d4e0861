"""Image output on the GPU (fr_resolve_rgba8 / fr_export_png) against the
oracle's restatement of the reference's ExportPNG, which is pinned to the
reference's own PNG files: exact on the GPU's resolved image; against the
reference's PNG of the golden runs, within one level where the images
themselves differ by FP32 summation order."""
import numpy as np
import pytest

from conftest import GOLDEN_SCENES, load_golden
from pngread import decode_png

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('name', sorted(GOLDEN_SCENES))
def test_export_matches_reference(name, tmp_path):
    from export_png import export_rgba8
    from frsppm import abi
    gold = load_golden(name)
    with abi.Renderer(GOLDEN_SCENES[name](), int(gold['photons']), alpha=0.9, radius=0.015) as r:
        r.iterate(int(gold['iters']))
        img = r.resolve()
        px = r.resolve_rgba8()
        np.testing.assert_array_equal(px, export_rgba8(img, r.width, r.height))
        diff = np.abs(px.astype(np.int32) - gold['image_png'].astype(np.int32))
        assert diff.max() <= 1 and (diff > 0).mean() < 0.01
        p = str(tmp_path / 'out.png')
        r.export_png(p)
        np.testing.assert_array_equal(decode_png(p), px)
