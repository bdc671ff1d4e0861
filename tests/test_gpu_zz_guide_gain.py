"""What the trained photon guide gains over plain light sampling, on the
small caustic box.  This is a statistical claim, so it sits in a file that
pytest collects after every deterministic GPU test (a run that stops at the
first failure has then checked all of parity first).

Each of three seeds (the guide's initial weights and, through fr_seek, the
random streams of both renders) gives a plain and a guided render of the same
iteration count.  Guided training is deterministic, so a seed's numbers are
the same on every run; the assertions are on the median over the seeds.
Both renders resolve with the standard estimate tau / (pi R^2 photons
emitted) (FR_FLAG_STANDARD_RESOLVE): the reference's own resolve scales each
pixel by its share of iterations with photons, which depends on the sampling
and so is not the same estimate for the two.  The reference image is a long
plain run whose random streams share no seed with the compared runs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEEDS = (1, 2, 3)


def _linear(img):
    """Resolve's pixels (radiance to the power 1/1.2) back to radiance."""
    return img[:, :3].astype(np.float64) ** 1.2


def _rel_mse(img, ref):
    a, b = _linear(img), _linear(ref)
    return float(np.mean((a - b) ** 2 / (b ** 2 + 1e-2)))


def test_trained_guide_gains_over_plain():
    from frsppm import abi, scenes
    scene = scenes.small_caustic()
    kw = dict(alpha=0.7, radius=0.01, flags=abi.FLAG_STANDARD_RESOLVE | abi.FLAG_END_DEGENERATE_PATHS)
    with abi.Renderer(scene, 100000, **kw) as ref:
        ref.seek(20000)
        ref.iterate(400)
        reference = ref.resolve()
    e_ref = _linear(reference).mean()
    iters, tail = 120, 20
    rows = []
    for seed in SEEDS:
        m_plain = m_guided = 0
        with abi.Renderer(scene, 50000, **kw) as plain, \
                abi.Renderer(scene, 50000, guide=True, guide_seed=seed, **kw) as guided:
            plain.seek(1000 * seed)
            guided.seek(1000 * seed)
            plain.iterate(iters - tail)
            guided.iterate(iters - tail)
            for _ in range(tail):
                plain.iterate(1)
                guided.iterate(1)
                m_plain += int(plain.read_gather()[0].sum())
                m_guided += int(guided.read_gather()[0].sum())
            useful = float((guided.guide_importance() > 0).mean())
            img_plain, img_guided = plain.resolve(), guided.resolve()
        rows.append(dict(seed=seed, m_ratio=m_guided / max(m_plain, 1), useful=useful,
                         e_plain=_rel_mse(img_plain, reference), e_guided=_rel_mse(img_guided, reference),
                         energy_plain=_linear(img_plain).mean() / e_ref,
                         energy_guided=_linear(img_guided).mean() / e_ref))
    for r in rows:
        print('seed %(seed)d: pairs guided/plain %(m_ratio).2f, useful %(useful).4f, relMSE plain %(e_plain).4f '
              'guided %(e_guided).4f, energy plain %(energy_plain).3f guided %(energy_guided).3f' % r)
    med = {k: float(np.median([r[k] for r in rows])) for k in rows[0] if k != 'seed'}
    # Photon-hitpoint pairs per iteration once trained and the share of paths
    # that reached a hitpoint (plain: about 0.1%).
    assert med['m_ratio'] > 4.0, rows
    assert med['useful'] > 0.005, rows
    # The guided estimate stays unbiased: the same energy as the reference.
    for r in rows:
        assert abs(r['energy_guided'] - 1.0) < 0.1 and abs(r['energy_plain'] - 1.0) < 0.1, r
    # The error at the same iteration count.
    assert med['e_guided'] < 0.7 * med['e_plain'], rows
