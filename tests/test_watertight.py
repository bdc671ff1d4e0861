"""The precision mode's watertight triangle test (Woop, Benthin and Wald,
JCGT 2(1), 2013) in the oracle (oracle/port), on the CPU:

* rays from inside a closed mesh aimed exactly at its shared vertices and
  edge midpoints never pass between triangles (every one hits the mesh);
* on the golden fixtures' rays it picks the same facets as the reference's
  Moller-Trumbore test except on a small share of rays (printed: the
  mismatch rate), and where both hit the same facet the distances agree to
  float rounding."""
import numpy as np
import pytest

from conftest import GOLDEN_SCENES, load_golden
from watertight_cases import closed_mesh_scene, edge_rays


def test_watertight_closes_shared_edges():
    import port_abi
    scene, V, F = closed_mesh_scene()
    rays = edge_rays(V, F)
    with port_abi.PortRenderer(scene, 1000) as mt, port_abi.PortRenderer(scene, 1000, watertight=True) as wt:
        f_mt, _ = mt.trace_closest(rays)
        f_wt, tuv = wt.trace_closest(rays)
    sphere = len(F)
    print('edge/vertex rays: %d; misses Moller-Trumbore %d, watertight %d'
          % (len(rays), int((f_mt < 0).sum()), int((f_wt < 0).sum())))
    assert (f_wt >= 0).all() and (f_wt < sphere).all()
    assert np.isfinite(tuv).all() and (tuv[:, 0] > 0).all()


@pytest.mark.parametrize('name', sorted(GOLDEN_SCENES))
def test_watertight_against_moller_trumbore_on_fixture_rays(name):
    import port_abi
    gold = load_golden(name)
    rays = gold['rays']
    with port_abi.PortRenderer(GOLDEN_SCENES[name](), int(gold['photons']), watertight=True) as wt:
        f, tuv = wt.trace_closest(rays)
        anyh = wt.trace_any(gold['any_rays'])
    ref_f, ref_tuv = gold['hit_facet'], gold['hit_tuv']
    diff = f != ref_f
    print('%s: %d rays, facet differs from the reference on %d (%.3f%%); any-hit differs on %d of %d'
          % (name, len(rays), int(diff.sum()), 100.0 * diff.mean(), int((anyh != gold['any_hit']).sum()),
             len(anyh)))
    assert diff.mean() < 0.005
    same = ~diff & (f >= 0)
    np.testing.assert_allclose(tuv[same, 0], ref_tuv[same, 0], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(tuv[same, 1:], ref_tuv[same, 1:], atol=1e-4)
    assert (anyh != gold['any_hit']).mean() < 0.005
