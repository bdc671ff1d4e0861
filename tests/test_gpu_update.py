"""fr_update against the reference's N/tau/R update (SPPM.cpp:444-449): fed the
reference's own per-hitpoint photon counts and flux sums of each golden
iteration, the state must reach the reference's N, R and NumGather bit for
bit and its tau within FP32 rounding (tau is FP64 here)."""
import numpy as np
import pytest

from conftest import GOLDEN_SCENES, load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('name', sorted(GOLDEN_SCENES))
def test_update_matches_reference(name):
    from frsppm import abi
    gold = load_golden(name)
    with abi.Renderer(GOLDEN_SCENES[name](), int(gold['photons']), alpha=0.9, radius=0.015) as r:
        for s in range(1, int(gold['iters']) + 1):
            r.update(gold['it%d_gather_m' % s], gold['it%d_gather_phi' % s])
            st = r.read_state()
            np.testing.assert_array_equal(st['n'], gold['it%d_sp_n' % s])
            np.testing.assert_array_equal(st['r'], gold['it%d_sp_r' % s])
            np.testing.assert_array_equal(st['g'], gold['it%d_sp_g' % s])
            ref = gold['it%d_sp_rad' % s]
            assert np.abs(st['tau'] - ref).max() <= 1e-5 * np.abs(ref).max() + 1e-30
        m, phi = r.read_gather()
        np.testing.assert_array_equal(m, gold['it%d_gather_m' % int(gold['iters'])])


def test_update_leaves_pixels_without_photons():
    from frsppm import abi, scenes
    with abi.Renderer(scenes.cornell_box(width=16, height=16), 1000, alpha=0.7, radius=0.02) as r:
        before = r.read_state()
        m = np.zeros(256, np.int32)
        m[5] = 3
        phi = np.zeros((256, 3), np.float32)
        phi[5] = (1.0, 2.0, 3.0)
        r.update(m, phi)
        after = r.read_state()
        keep = np.arange(256) != 5
        for k in ('n', 'r', 'g'):
            np.testing.assert_array_equal(after[k][keep], before[k][keep])
        assert after['g'][5] == 1 and after['n'][5] == int(np.float32(3) * np.float32(0.7))
        np.testing.assert_allclose(after['tau'][5], np.array([1.0, 2.0, 3.0]) * (2.1 / 3.0), rtol=1e-6)
        assert after['r'][5] == np.float32(0.02) * np.sqrt(np.float32(2.1) / np.float32(3.0), dtype=np.float32)


@pytest.mark.parametrize('name', sorted(GOLDEN_SCENES))
def test_update_dev_matches_update(name):
    """fr_update_dev (device inputs) reaches the state fr_update reaches."""
    import torch
    from frsppm import abi
    gold = load_golden(name)
    mk = lambda: abi.Renderer(GOLDEN_SCENES[name](), int(gold['photons']), alpha=0.9, radius=0.015)
    with mk() as a, mk() as b:
        for s in range(1, int(gold['iters']) + 1):
            m = gold['it%d_gather_m' % s]
            phi = gold['it%d_gather_phi' % s]
            a.update(m, phi)
            md = torch.from_numpy(np.ascontiguousarray(m, np.int32)).cuda()
            p4 = np.zeros((len(m), 4), np.float32)
            p4[:, :3] = phi.reshape(-1, 3)
            pd = torch.from_numpy(p4).cuda()
            torch.cuda.synchronize()
            b.update_dev(md.data_ptr(), pd.data_ptr())
            sa, sb = a.read_state(), b.read_state()
            for k in ('n', 'r', 'g', 'tau'):
                np.testing.assert_array_equal(sa[k], sb[k])
