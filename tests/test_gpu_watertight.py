"""FR_FLAG_WATERTIGHT on the GPU against the oracle's watertight test
(oracle/port), bit for bit: closest hits (facet, t, u, v) and any hits on
rays aimed exactly at a closed mesh's shared vertices and edges and on the
golden fixtures' rays; the reference's Moller-Trumbore mode on the same
edge rays (misses included).  Whole renders in the watertight mode are
compared with the oracle in test_gpu_oracle_parity.py."""
import numpy as np
import pytest

from conftest import GOLDEN_SCENES, load_golden
from watertight_cases import closed_mesh_scene, edge_rays

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('watertight', [False, True])
def test_edge_rays_match_oracle(watertight):
    import port_abi
    from frsppm import abi
    scene, V, F = closed_mesh_scene()
    rays = edge_rays(V, F)
    flags = abi.FLAG_WATERTIGHT if watertight else 0
    with abi.Renderer(scene, 1000, flags=flags) as g, port_abi.PortRenderer(scene, 1000, watertight=watertight) as c:
        fg, tg = g.trace_closest(rays)
        fc, tc = c.trace_closest(rays)
    np.testing.assert_array_equal(fg, fc)
    h = fc >= 0
    np.testing.assert_array_equal(tg[h], tc[h])
    if watertight:
        assert h.all()


@pytest.mark.parametrize('name', sorted(GOLDEN_SCENES))
def test_fixture_rays_match_oracle(name):
    import port_abi
    from frsppm import abi
    gold = load_golden(name)
    scene = GOLDEN_SCENES[name]()
    with abi.Renderer(scene, 1000, flags=abi.FLAG_WATERTIGHT) as g, \
            port_abi.PortRenderer(scene, 1000, watertight=True) as c:
        fg, tg = g.trace_closest(gold['rays'])
        fc, tc = c.trace_closest(gold['rays'])
        np.testing.assert_array_equal(fg, fc)
        h = fc >= 0
        np.testing.assert_array_equal(tg[h], tc[h])
        np.testing.assert_array_equal(g.trace_any(gold['any_rays']), c.trace_any(gold['any_rays']))
