"""GPU path against the oracle (the CPU restatement pinned to the reference)
on larger seeded cases than the golden fixtures hold."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {
    # name: (scene factory, photons, iterations, alpha, radius[, options])
    # options: fix_stale (FR_FLAG_FIX_STALE_PHOTON_SLOT), watertight
    # (FR_FLAG_WATERTIGHT), each against the oracle's switch.
    'cornell96': (lambda s: s.cornell_box(width=96, height=96), 20000, 4, 0.7, 0.02),
    # The Cornell-box configuration at full size: 256^2 pinhole, 100k paths.
    'cornell256_100k': (lambda s: s.cornell_box(), 100000, 2, 0.7, 0.02),
    # FR_FLAG_FIX_STALE_PHOTON_SLOT against the oracle's switch.
    'cornell96_fixstale': (lambda s: s.cornell_box(width=96, height=96), 20000, 3, 0.7, 0.02, {'fix_stale': True}),
    # The precision mode's watertight triangle test.
    'cornell96_watertight': (lambda s: s.cornell_box(width=96, height=96), 20000, 3, 0.7, 0.02,
                             {'watertight': True}),
    # N kept as a float (FR_FLAG_FLOAT_PHOTON_COUNT), not the reference's truncated int.
    'cornell96_floatcount': (lambda s: s.cornell_box(width=96, height=96), 20000, 4, 0.7, 0.02,
                             {'float_count': True}),
    'mixed128x72_watertight': (lambda s: s.mixed_materials(width=128, height=72, n_spheres=24, field_n=48,
                                                           tex_size=128, light_tex=64, n_lat=12, n_lon=16,
                                                           extent=0.8, aperture=0.05),
                               20000, 3, 0.7, 0.02, {'watertight': True}),
    'mixed128x72': (lambda s: s.mixed_materials(width=128, height=72, n_spheres=24, field_n=48, tex_size=128,
                                                light_tex=64, n_lat=12, n_lon=16, extent=0.8, aperture=0.05),
                    20000, 3, 0.7, 0.02),
    # The caustic box (glass spheres, slit) and the large scene's construction
    # (displaced geodesic spheres, instanced and flattened), small.
    'caustic96': (lambda s: s.small_caustic(), 20000, 3, 0.7, 0.01),
    'large64x36': (lambda s: s.small_large_scene(), 20000, 3, 0.7, 0.02),
    # All eight surface types (the demo's BiMetal, Glass, GlossTransmit and
    # DiffuseTransmit beside the four of the configs).
    'demo128x72': (lambda s: s.demo_materials(width=128, height=72, n_spheres=32, field_n=48, tex_size=128,
                                              light_tex=64, extent=0.8), 20000, 3, 0.7, 0.02),
    # With an environment map: eye paths go on after their hitpoints.
    'mixed128x72_ibl': (lambda s: s.with_sky(s.mixed_materials(width=128, height=72, n_spheres=24, field_n=48,
                                                               tex_size=128, light_tex=64, n_lat=12, n_lon=16,
                                                               extent=0.8, aperture=0.05), 77),
                        20000, 3, 0.7, 0.02),
}


def _scene(name):
    from frsppm import scenes
    return CASES[name][0](scenes)


def _image_close(ig, ic):
    """Per pixel and channel |gpu - oracle| <= 1e-4 |oracle| + 1e-7 max: the
    flux sums differ only by float summation order and by ulps of the
    transcendental functions, relative to each pixel's own value; the
    absolute floor (1e-7 of the image maximum) covers pixels near zero."""
    a, b = ig[:, :3].astype(np.float64), ic[:, :3].astype(np.float64)
    bad = np.abs(a - b) > 1e-4 * np.abs(b) + 1e-7 * np.abs(b).max()
    assert not bad.any(), (int(bad.sum()), float((np.abs(a - b) / np.maximum(np.abs(b), 1e-30))[bad].max()))


def _compare_iteration(g, c, scene):
    hg, hc = g.read_hitpoints(), c.read_hitpoints()
    np.testing.assert_array_equal(hg['type'] == 1, hc['type'] == 1)
    h = hc['type'] == 1
    np.testing.assert_array_equal(hg['facet'][h], hc['facet'][h])
    np.testing.assert_array_equal(hg['pos'][h], hc['pos'][h])
    pg, path_g, slot_g = g.compacted_photons()
    pc, path_c, slot_c = c.compacted_photons()
    np.testing.assert_array_equal(path_g, path_c)
    np.testing.assert_array_equal(slot_g, slot_c)
    np.testing.assert_array_equal(pg[:, :3], pc[:, :3])
    mg, _ = g.read_gather()
    mc, _ = c.read_gather()
    np.testing.assert_array_equal(mg, mc)
    sg, sc = g.read_state(), c.read_state()
    np.testing.assert_array_equal(sg['n'], sc['n'])
    np.testing.assert_array_equal(sg['r'], sc['r'])
    np.testing.assert_array_equal(sg['g'], sc['g'])
    if scene.get('ibl') is not None:
        np.testing.assert_array_equal(hg['type'], hc['type'])
        lg, tg, ng = g.read_direct()
        lc, tc, nc = c.read_direct()
        np.testing.assert_array_equal(ng, nc)
        for a, b in ((lg, lc), (tg, tc)):
            assert np.abs(a - b).max() <= 1e-4 * np.abs(b).max() + 1e-30
    assert np.abs(sg['tau'] - sc['tau']).max() <= 1e-4 * np.abs(sc['tau']).max()


@pytest.mark.parametrize('name', sorted(CASES))
def test_gpu_matches_oracle(name):
    import port_abi
    from frsppm import abi
    _, photons, iters, alpha, radius = CASES[name][:5]
    opt = CASES[name][5] if len(CASES[name]) > 5 else {}
    fix, wt, fc = opt.get('fix_stale', False), opt.get('watertight', False), opt.get('float_count', False)
    scene = _scene(name)
    flags = ((abi.FLAG_FIX_STALE_PHOTON_SLOT if fix else 0) | (abi.FLAG_WATERTIGHT if wt else 0) |
             (abi.FLAG_FLOAT_PHOTON_COUNT if fc else 0))
    with abi.Renderer(scene, photons, alpha=alpha, radius=radius, flags=flags) as g, \
            port_abi.PortRenderer(scene, photons, alpha=alpha, radius=radius, fix_stale=fix, watertight=wt,
                                  float_count=fc) as c:
        for s in range(iters):
            g.iterate(1)
            c.iterate(1)
            _compare_iteration(g, c, scene)
        ig, ic = g.resolve(), c.resolve()
    _image_close(ig, ic)


# The mixed-materials, caustic and large-scene configurations at full size:
# 1280x720 thin lens with 1M photon paths (997,444 triangles, textures), the
# 1024^2 caustic box with 2M photon paths (198,936 triangles), and the large
# scene (20,000,004 triangles, 4096^2 textures, 3840x2160 thin lens) with 8M
# photon paths, without its learned guide (the oracle has none).
FULL = {
    'mixed_materials_1280x720_1M': (lambda s: s.mixed_materials(), 1_000_000, 2, 0.7, 0.02),
    'caustic_box_1024_2M': (lambda s: s.caustic_box(), 2_000_000, 1, 0.7, 0.01),
    'large_scene_3840x2160_8M': (lambda s: s.large_scene(), 8_000_000, 1, 0.7, 0.02),
}


@pytest.mark.parametrize('name', sorted(FULL))
def test_gpu_matches_oracle_full_size(name):
    import port_abi
    from frsppm import abi, scenes
    factory, photons, iters, alpha, radius = FULL[name]
    scene = factory(scenes)
    with abi.Renderer(scene, photons, alpha=alpha, radius=radius) as g, \
            port_abi.PortRenderer(scene, photons, alpha=alpha, radius=radius) as c:
        for s in range(iters):
            g.iterate(1)
            c.iterate(1)
            _compare_iteration(g, c, scene)
        ig, ic = g.resolve(), c.resolve()
    _image_close(ig, ic)


def test_gpu_radius_query_matches_oracle_large():
    """Counts at 200k photons / 50k hitpoints on surfaces, against the oracle's kd-tree."""
    import port_abi
    from frsppm import abi, scenes
    rng = np.random.Generator(np.random.PCG64(11))
    ph = rng.uniform(-2, 2, (200_000, 3)).astype(np.float32)
    ph[:, 1] = rng.choice([0.0, 0.3, 1.7], len(ph))
    hp = rng.uniform(-2, 2, (50_000, 3)).astype(np.float32)
    hp[:, 1] = rng.choice([0.0, 0.3, 1.7], len(hp))
    R = rng.uniform(0.002, 0.05, len(hp)).astype(np.float32)
    with abi.Renderer(scenes.cornell_box(width=8, height=8), 16) as r:
        got, _ = r.radius_query(hp, R, ph, 0.04)
    np.testing.assert_array_equal(got, port_abi.radius_count(hp, R, ph))
