"""bench.py's traversal work figures are the ones the reference's harness
measured (tests/golden/make_traversal_work.py)."""
import json
import os

from conftest import GOLDEN, REPO


def test_traversal_work_matches_the_measurement():
    import importlib.util
    spec = importlib.util.spec_from_file_location('bench_mod', os.path.join(REPO, 'bench.py'))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    with open(os.path.join(GOLDEN, 'traversal_work_mixed.json')) as f:
        w = json.load(f)
    for k in ('eye', 'photon'):
        assert bench.TRAVERSAL_FP32_OPS_PER_RAY[k] == w[k]['fp32_ops_per_ray']
        assert w[k]['rays'] > 100_000
        assert w[k]['fp32_ops_per_ray'] == 168.0 * w[k]['mean_nodes_V'] + 40.0 * w[k]['mean_leaf_tests_X']
