"""The photon guide's CPU oracle (oracle/guide_ref.py): its analytic gradient of
the training loss against central finite differences of the loss, in float64."""
import numpy as np


def _case(seed, n):
    import guide_ref as G
    rng = np.random.Generator(np.random.PCG64(seed))
    p = rng.normal(0.0, 0.3, G.N_PARAMS)
    p[G.OFF_W4 + G.OUT * G.HID:G.OFF_B4] = 0.0
    p[G.OFF_B4 + G.OUT:] = 0.0
    x = np.concatenate([rng.uniform(-1, 1, (n, 3)), rng.uniform(0, 1, (n, 2))], 1)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    I = rng.exponential(1.0, n) * (rng.random(n) > 0.2)
    return p, np.concatenate([x, d, I[:, None]], 1)


def test_analytic_gradient_matches_finite_differences():
    import guide_ref as G
    p, smp = _case(3, 16)
    g, wsum = G.gradient(p, smp, bf16_rounding=False)
    assert abs(wsum - smp[:, 8].sum()) < 1e-9
    rng = np.random.Generator(np.random.PCG64(4))
    used = np.r_[G.OFF_W1:G.OFF_W4 + G.OUT * G.HID, G.OFF_B4:G.OFF_B4 + G.OUT]
    for k in rng.choice(used, 60, replace=False):
        h = 1e-6 * max(1.0, abs(p[k]))
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (G.loss(pp, smp) - G.loss(pm, smp)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-4 * max(1.0, abs(fd)), (k, fd, g[k])


def test_bf16_rounding_stays_close_to_exact():
    import guide_ref as G
    p, smp = _case(5, 256)
    ge, _ = G.gradient(p, smp, bf16_rounding=False)
    gb, _ = G.gradient(p, smp, bf16_rounding=True)
    assert np.linalg.norm(gb - ge) <= 0.05 * np.linalg.norm(ge)
