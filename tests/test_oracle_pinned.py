"""Pins the oracle (oracle/port, the CPU restatement) to the reference's own
outputs: the golden fixtures were made by running the reference's SPPM code
(tests/golden/make_golden.py).  Runs on CPU only."""
import numpy as np
import pytest

from conftest import GOLDEN_SCENES, load_golden

NAMES = sorted(GOLDEN_SCENES)


@pytest.fixture(scope='module')
def port():
    import port_abi
    port_abi.load()
    return port_abi


def test_philox_known_answers(port):
    # Known-answer vectors of Philox4x32-10 (Random123 test data).
    cases = [([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
             ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
             ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
              [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1])]
    for ctr, key, want in cases:
        assert list(port.philox(ctr, key)) == want


@pytest.mark.parametrize('name', NAMES)
def test_oracle_hits_match_reference(port, name):
    gold = load_golden(name)
    with port.PortRenderer(GOLDEN_SCENES[name](), int(gold['photons'])) as r:
        f, tuv = r.trace_closest(gold['rays'])
        np.testing.assert_array_equal(f, gold['hit_facet'])
        hit = f >= 0
        np.testing.assert_array_equal(tuv[hit], gold['hit_tuv'][hit])
        np.testing.assert_array_equal(r.trace_any(gold['any_rays']), gold['any_hit'])


@pytest.mark.parametrize('name', NAMES)
def test_oracle_iterations_match_reference(port, name):
    gold = load_golden(name)
    with port.PortRenderer(GOLDEN_SCENES[name](), int(gold['photons'])) as r:
        for s in range(1, int(gold['iters']) + 1):
            r.iterate(1)
            hp = r.read_hitpoints()
            t = gold['it%d_hp_type' % s]
            np.testing.assert_array_equal(hp['type'] == 1, t == 1)
            h = t == 1
            for k in ('facet', 'pos', 'nrm', 'out', 'w', 'rough'):
                np.testing.assert_array_equal(hp[k][h], gold['it%d_hp_%s' % (s, k)][h])
            ph, path, slot = r.compacted_photons()
            np.testing.assert_array_equal(path, gold['it%d_ph_path' % s])
            np.testing.assert_array_equal(slot, gold['it%d_ph_slot' % s])
            np.testing.assert_array_equal(ph, gold['it%d_ph' % s])
            m, phi = r.read_gather()
            np.testing.assert_array_equal(m, gold['it%d_gather_m' % s])
            ref = gold['it%d_gather_phi' % s]
            # The reference sums in kd-tree order; only the order differs.
            assert np.abs(phi - ref).max() <= 1e-5 * np.abs(ref).max()
            st = r.read_state()
            np.testing.assert_array_equal(st['n'], gold['it%d_sp_n' % s])
            np.testing.assert_array_equal(st['r'], gold['it%d_sp_r' % s])
            np.testing.assert_array_equal(st['g'], gold['it%d_sp_g' % s])
            assert np.abs(st['tau'] - gold['it%d_sp_rad' % s]).max() <= 1e-5 * np.abs(gold['it%d_sp_rad' % s]).max()
            if 'it%d_hp_dl' % s in gold:  # environment light: types, direct light, sums, counts
                np.testing.assert_array_equal(hp['type'], t)
                last, tot, cnt = r.read_direct()
                np.testing.assert_array_equal(last, gold['it%d_hp_dl' % s])
                np.testing.assert_array_equal(tot, gold['it%d_sp_dl' % s])
                np.testing.assert_array_equal(cnt, gold['it%d_sp_ndl' % s])
        img = r.resolve()
    assert np.abs(img - gold['image']).max() <= 1e-5 * np.abs(gold['image']).max()


def test_oracle_radius_query_matches_exhaustive(port):
    rng = np.random.Generator(np.random.PCG64(7))
    ph = rng.uniform(0, 1, (5000, 3)).astype(np.float32)
    ph[:, 1] = rng.choice([0.0, 0.25], 5000)  # coplanar photons, as SPPM deposits them
    hp = rng.uniform(0, 1, (400, 3)).astype(np.float32)
    hp[:, 1] = rng.choice([0.0, 0.25], 400)
    R = rng.uniform(0.01, 0.08, 400).astype(np.float32)
    got = port.radius_count(hp, R, ph)
    f32 = np.float32
    for i in range(len(hp)):
        inside = np.all((hp[i] - R[i] * f32(1) <= ph) & (hp[i] + R[i] * f32(1) >= ph), axis=1)
        d = ph - hp[i]
        n2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        assert got[i] == int((inside & (n2 < R[i] * R[i])).sum())
