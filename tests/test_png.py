"""fr_write_png (host only): the file is a PNG that decodes to the bytes given."""
import numpy as np

from pngread import decode_png


def test_write_png_roundtrip(tmp_path):
    from frsppm import abi
    rng = np.random.Generator(np.random.PCG64(7))
    for h, w in ((1, 1), (3, 5), (64, 48), (300, 250)):   # 300 rows x 1001 B: more than one stored block
        img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
        p = str(tmp_path / ('i%dx%d.png' % (h, w)))
        abi.write_png(p, img)
        np.testing.assert_array_equal(decode_png(p), img)


def test_write_png_rejects_bad_size(tmp_path):
    from frsppm import abi
    import pytest
    with pytest.raises(RuntimeError):
        abi.write_png(str(tmp_path / 'x.png'), np.zeros((0, 4, 4), np.uint8))


def test_export_restatement_matches_reference_png():
    """The oracle's ExportPNG restatement on the reference's float image gives
    the reference's own PNG pixels (golden fixtures)."""
    from conftest import GOLDEN_SCENES, load_golden
    from export_png import export_rgba8
    for name in GOLDEN_SCENES:
        gold = load_golden(name)
        h, w = gold['image_png'].shape[:2]
        np.testing.assert_array_equal(export_rgba8(gold['image'], w, h), gold['image_png'])
