"""Traversal work of the mixed-materials workload on the reference's own BVH.

    python tests/golden/make_traversal_work.py

The CPU restatement (oracle/port) runs one iteration of the mixed-materials
scene (frsppm.scenes.mixed_materials: 997,444 triangles, 1280x720, 1M photon
paths) and keeps every 10th closest-hit ray it traces, eye and photon rays
alike (the GPU traces the same rays: its hits are the restatement's).  The
reference's harness (oracle/_ref/frref, built from the reference sources)
loads the same scene through Scene::CreateScene and runs the reference's
closest-hit loop (N_BVH8::findClosestElement, bvh8.h:568-641) on those rays,
counting per ray the internal nodes whose child boxes it tests (V) and the
leaves whose triangle it tests (X).  The work per ray is 168 V + 40 X FP32
operations (21 per child slab test, 8 children; about 40 per Moller-Trumbore
test, Intersect.cpp:67-89, 515-553).  Writes traversal_work_mixed.json next
to this file; bench.py carries the same figures (tests/test_bench_contract.py
keeps them equal).
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, 'friendsrender-r-public_gb300'))
sys.path.insert(0, os.path.join(REPO, 'oracle'))
from frsppm import objio, scenes  # noqa: E402

FRREF = os.path.join(REPO, 'oracle', '_ref', 'frref')
PHOTONS, STRIDE, CAP = 1_000_000, 10, 400_000


def main():
    import port_abi
    scene = scenes.mixed_materials()
    t0 = time.time()
    with port_abi.PortRenderer(scene, PHOTONS, alpha=0.7, radius=0.02) as p:
        p.sample_rays(STRIDE, CAP)
        p.iterate(1)
        rays, passes = p.ray_sample()
    print('sampled %d rays (%.0f s)' % (len(rays), time.time() - t0), flush=True)
    with tempfile.TemporaryDirectory() as d:
        objio.write_scene(scene, d)
        objio.write_materials_table(scene, os.path.join(d, 'materials.txt'))
        objio.write_camera(scene, os.path.join(d, 'camera.txt'))
        rays.tofile(os.path.join(d, 'rays.bin'))
        t0 = time.time()
        r = subprocess.run([FRREF, d, 'count', os.path.join(d, 'rays.bin'), d], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('frref count failed (%d): %s' % (r.returncode, r.stderr[-2000:]))
        vx = np.load(os.path.join(d, 'visits.npy')).astype(np.float64)
        print('counted (%.0f s)' % (time.time() - t0), flush=True)

    def summary(sel):
        v, x = vx[sel, 0].mean(), vx[sel, 1].mean()
        return {'rays': int(sel.sum()), 'mean_nodes_V': v, 'mean_leaf_tests_X': x,
                'fp32_ops_per_ray': 168.0 * v + 40.0 * x}

    out = {'workload': 'mixed materials: 997,444 triangles, 1280x720, 1M photon paths, iteration 1',
           'sample': 'every %dth closest-hit ray of the CPU restatement' % STRIDE,
           'work': '168 V + 40 X FP32 operations per ray on the reference BVH (bvh8.h:568-641)',
           'all': summary(np.ones(len(vx), bool)), 'eye': summary(passes == 0), 'photon': summary(passes == 1)}
    with open(os.path.join(HERE, 'traversal_work_mixed.json'), 'w') as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == '__main__':
    sys.exit(main())
