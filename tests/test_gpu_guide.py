"""The learned photon-emission guide on the GPU.

* Its training gradient (tensor-core forward and backward) against the CPU
  oracle's restatement of the same network and loss (oracle/guide_ref.py),
  with the oracle rounding to bfloat16 where the kernels do.
* A guided render stays a valid SPPM render (finite, same hitpoints as plain).
* Its training is deterministic (the same network bit for bit on a rerun).
* What the trained network gains over plain emission is measured in
  test_gpu_zz_guide_gain.py, collected after every deterministic GPU test.
* fr_seek, which gives the long reference render random streams of its own.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oracle_case(seed, n):
    import guide_ref as G
    rng = np.random.Generator(np.random.PCG64(seed))
    p = rng.normal(0.0, 0.25, G.N_PARAMS).astype(np.float32)
    p[G.OFF_W4 + G.OUT * G.HID:G.OFF_B4] = 0.0
    p[G.OFF_B4 + G.OUT:] = 0.0
    x = np.concatenate([rng.uniform(-1, 1, (n, 3)), rng.uniform(0, 1, (n, 2))], 1)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    I = rng.exponential(1.0, n) * (rng.random(n) > 0.1)
    return p, np.concatenate([x, d, I[:, None]], 1).astype(np.float32)


@pytest.mark.parametrize('n', [100, 128, 1000])
def test_guide_gradient_matches_oracle(n):
    import guide_ref as G
    from frsppm import abi, scenes
    p, smp = _oracle_case(n, n)
    with abi.Renderer(scenes.cornell_box(width=16, height=16), 2048, guide=True, guide_batch=2048) as r:
        r.set_guide_params(p)
        np.testing.assert_array_equal(r.guide_params(), p)
        g_gpu, ws_gpu = r.guide_gradient(smp)
    g_ref, ws_ref = G.gradient(p.astype(np.float64), smp.astype(np.float64), bf16_rounding=True)
    sel = np.ones(G.N_PARAMS, bool)
    sel[G.OFF_W4 + G.OUT * G.HID:G.OFF_B4] = False
    sel[G.OFF_B4 + G.OUT:] = False
    assert np.abs(g_gpu[~sel]).max() == 0.0
    a, b = g_gpu[sel].astype(np.float64), g_ref[sel]
    assert abs(ws_gpu - ws_ref) <= 1e-5 * ws_ref
    assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b)
    assert a @ b / (np.linalg.norm(a) * np.linalg.norm(b)) > 0.9995
    # and each layer's block on its own
    for lo, hi in ((G.OFF_W1, G.OFF_W2), (G.OFF_W2, G.OFF_W3), (G.OFF_W3, G.OFF_W4), (G.OFF_W4, G.N_PARAMS)):
        m = sel[lo:hi]
        assert np.linalg.norm(g_gpu[lo:hi][m] - g_ref[lo:hi][m]) <= 3e-2 * np.linalg.norm(g_ref[lo:hi][m])


def test_guided_render_is_valid():
    from frsppm import abi, scenes
    scene = scenes.small_caustic()
    with abi.Renderer(scene, 40000, alpha=0.7, radius=0.01) as plain, \
            abi.Renderer(scene, 40000, alpha=0.7, radius=0.01, guide=True) as guided:
        plain.iterate(3)
        guided.iterate(3)
        hp, hg = plain.read_hitpoints(), guided.read_hitpoints()
        np.testing.assert_array_equal(hp['type'], hg['type'])      # the eye pass is the same
        img = guided.resolve()
        assert np.isfinite(img).all()
        p = guided.guide_params()
        assert np.isfinite(p).all()


def test_guided_training_is_deterministic():
    """Two guided renders of the same scene and seed train the same network
    bit for bit: importance is summed in fixed point, samples are taken in
    path order and the per-CTA gradient sums are added in CTA order."""
    from frsppm import abi, scenes
    scene = scenes.small_caustic()
    kw = dict(alpha=0.7, radius=0.01, guide=True, flags=abi.FLAG_END_DEGENERATE_PATHS)
    with abi.Renderer(scene, 50000, **kw) as a, abi.Renderer(scene, 50000, **kw) as b:
        for _ in range(6):
            a.iterate(1)
            b.iterate(1)
            np.testing.assert_array_equal(a.guide_importance(), b.guide_importance())
            np.testing.assert_array_equal(a.guide_params(), b.guide_params())
        assert (a.guide_importance() > 0).any()
        np.testing.assert_array_equal(a.read_state()['n'], b.read_state()['n'])


def test_seek_moves_random_streams():
    """fr_seek(s) on a fresh context: its first iteration is the iteration
    s + 1 of an unmoved context (same hitpoints), and the checkpoint keeps it."""
    from frsppm import abi, scenes
    scene = scenes.small_caustic(width=32, height=32)
    with abi.Renderer(scene, 5000, radius=0.01) as a, abi.Renderer(scene, 5000, radius=0.01) as b, \
            abi.Renderer(scene, 5000, radius=0.01) as c:
        a.iterate(3)
        b.seek(2)
        b.iterate(1)
        np.testing.assert_array_equal(a.read_hitpoints()['pos'], b.read_hitpoints()['pos'])
        c.load_state(b.save_state())
        a.iterate(1)
        c.iterate(1)
        np.testing.assert_array_equal(a.read_hitpoints()['pos'], c.read_hitpoints()['pos'])
        with pytest.raises(RuntimeError):
            b.seek(5)  # iterations already run
