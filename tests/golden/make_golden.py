"""Make the golden fixtures under tests/golden/ by running the reference's own
SPPM code (oracle/_ref/frref, built by oracle/ref/Makefile from the reference
sources) on small seeded scenes.

    python tests/golden/make_golden.py

Each fixture <name>.npz holds, for a scene from frsppm.scenes:
  scene_sha                 digest of the scene arrays the fixture was made from
  rays, hit_facet, hit_tuv  closest-hit queries (Scene::GetOneFacetFromRay)
  any_rays, any_hit         any-hit queries (N_BVH8::AnyHit)
  it{s}_*                   per iteration s = 1..iters: hitpoints, compacted
                            photons (with path and slot), gather M and flux,
                            per-pixel state after the update
  image, meta               reconstructImageFromSharedPoints output and
                            [total photons, iterations, threads]
  image_png                 the reference's ExportPNG of that image, decoded
                            (height x width x RGBA8)
with the reference's ppm_Alpha = 0.9 and FirstRadius = 0.015 (SPPM.cpp:20-21).

caustic_step51_row780.npz: one row (780) of the hitpoints that the reference's
eye pass makes at step 51 on the full caustic scene (frsppm.scenes.caustic_box,
1024^2), where pixel 799031 gets a NaN weight from the reference's
rough-dielectric BSDF: hp_* as above, with scene_sha, step and row.  The render
mode dumps every step up to 51, about 3.6 GB in the working folder.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, 'friendsrender-r-public_gb300'))
from frsppm import objio, scenes  # noqa: E402

sys.path.insert(0, os.path.join(REPO, 'tests'))
from pngread import decode_png  # noqa: E402

FRREF = os.path.join(REPO, 'oracle', '_ref', 'frref')

FIXTURES = {
    # name: (scene factory, photons per iteration, iterations)
    'cornell32': (lambda: scenes.cornell_box(width=32, height=32), 2000, 3),
    'mixed48x32': (lambda: scenes.small_mixed(), 2000, 3),
    'mixed48x32_ibl': (lambda: scenes.small_mixed(ibl=True), 2000, 3),
    'demo48x32': (lambda: scenes.demo_materials(), 3000, 3),
}


def scene_sha(scene):
    h = hashlib.sha256()
    for k in ('pos', 'nrm', 'uv', 'mat'):
        h.update(np.ascontiguousarray(scene[k]).tobytes())
    for t in scene['textures']:
        h.update(np.ascontiguousarray(t).tobytes())
    if scene.get('ibl') is not None:
        h.update(b'ibl' + np.ascontiguousarray(scene['ibl']).tobytes())
    h.update(repr([sorted(m.items()) for m in scene['materials']]).encode())
    h.update(repr(sorted(scene['camera'].items())).encode())
    return h.hexdigest()


def query_rays(scene, n, seed):
    """Closest-hit rays: origins inside the scene bounds, uniform directions,
    plus the camera position toward random scene points."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lo, hi = scene['pos'].reshape(-1, 3).min(0), scene['pos'].reshape(-1, 3).max(0)
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    cam = np.asarray(scene['camera']['pos'])
    k = n // 4
    o[:k] = cam
    d[:k] = rng.uniform(lo, hi, (k, 3)) - cam
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d, np.ones((n, 1))], 1).astype(np.float32)


def any_rays(scene, n, seed):
    """Segments between two random points in the bounds: {org, dir, min_t, max_t}."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lo, hi = scene['pos'].reshape(-1, 3).min(0), scene['pos'].reshape(-1, 3).max(0)
    a = rng.uniform(lo, hi, (n, 3))
    b = rng.uniform(lo, hi, (n, 3))
    d = b - a
    L = np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([a, d / L, np.full((n, 1), 1e-4), L], 1).astype(np.float32)


def run(args):
    r = subprocess.run([FRREF] + args, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('frref %s failed: %s' % (' '.join(args), r.stderr))


def make(name, factory, photons, iters, out_dir=HERE):
    scene = factory()
    with tempfile.TemporaryDirectory() as d:
        objio.write_scene(scene, d)
        objio.write_materials_table(scene, os.path.join(d, 'materials.txt'))
        objio.write_camera(scene, os.path.join(d, 'camera.txt'))
        od = os.path.join(d, 'out')
        os.makedirs(od)
        run([d, 'facets', od])
        for k, ref in (('facet_pos', 'pos'), ('facet_nrm', 'nrm'), ('facet_uv', 'uv'), ('facet_attr', 'mat')):
            got = np.load(os.path.join(od, k + '.npy'))
            if not np.array_equal(got, scene[ref]):
                raise RuntimeError('%s: the reference loaded different %s' % (name, ref))
        rays = query_rays(scene, 4096, 1)
        rays.tofile(os.path.join(d, 'rays.bin'))
        run([d, 'trace', os.path.join(d, 'rays.bin'), od])
        arays = any_rays(scene, 4096, 2)
        arays.tofile(os.path.join(d, 'arays.bin'))
        run([d, 'any', os.path.join(d, 'arays.bin'), od])
        run([d, 'render', str(photons), str(iters), od])
        data = dict(scene_sha=np.array(scene_sha(scene)), photons=np.array(photons), iters=np.array(iters),
                    rays=rays, hit_facet=np.load(os.path.join(od, 'hit_facet.npy')),
                    hit_tuv=np.load(os.path.join(od, 'hit_tuv.npy')), any_rays=arays,
                    any_hit=np.load(os.path.join(od, 'any_hit.npy')),
                    image=np.load(os.path.join(od, 'image.npy')), meta=np.load(os.path.join(od, 'meta.npy')),
                    image_png=decode_png(os.path.join(od, 'image.png')))
        for s in range(1, iters + 1):
            for k in ('hp_type', 'hp_facet', 'hp_pos', 'hp_nrm', 'hp_out', 'hp_w', 'hp_rough', 'hp_dl', 'ph', 'ph_path',
                      'ph_slot', 'gather_m', 'gather_phi', 'sp_rad', 'sp_r', 'sp_n', 'sp_g', 'sp_dl', 'sp_ndl'):
                data['it%d_%s' % (s, k)] = np.load(os.path.join(od, 'it%d_%s.npy' % (s, k)))
    path = os.path.join(out_dir, name + '.npz')
    np.savez_compressed(path, **data)
    return path


CAUSTIC_STEP, CAUSTIC_ROW = 51, 780
HP_KEYS = ('hp_type', 'hp_facet', 'hp_pos', 'hp_nrm', 'hp_out', 'hp_w', 'hp_rough')


def caustic_row_fixture(scene, od, out_dir=HERE):
    """The fixture from a finished 'render 1000 51' output folder od."""
    W = scene['camera']['width']
    sl = slice(CAUSTIC_ROW * W, (CAUSTIC_ROW + 1) * W)
    data = dict(scene_sha=np.array(scene_sha(scene)), step=np.array(CAUSTIC_STEP), row=np.array(CAUSTIC_ROW))
    for k in HP_KEYS:
        data[k] = np.load(os.path.join(od, 'it%d_%s.npy' % (CAUSTIC_STEP, k)))[sl]
    path = os.path.join(out_dir, 'caustic_step%d_row%d.npz' % (CAUSTIC_STEP, CAUSTIC_ROW))
    np.savez_compressed(path, **data)
    return path


def make_caustic_row(out_dir=HERE, work=None):
    scene = scenes.caustic_box()
    with tempfile.TemporaryDirectory(dir=work) as d:
        objio.write_scene(scene, d)
        objio.write_materials_table(scene, os.path.join(d, 'materials.txt'))
        objio.write_camera(scene, os.path.join(d, 'camera.txt'))
        od = os.path.join(d, 'out')
        os.makedirs(od)
        run([d, 'render', '1000', str(CAUSTIC_STEP), od])
        return caustic_row_fixture(scene, od, out_dir)


if __name__ == '__main__':
    if not os.path.exists(FRREF):
        sys.exit('build the reference first: make -C oracle/ref')
    only = sys.argv[1:]
    for name, (factory, photons, iters) in FIXTURES.items():
        if only and name not in only:
            continue
        p = make(name, factory, photons, iters)
        print(p, os.path.getsize(p))
    if not only or 'caustic' in only:
        p = make_caustic_row()
        print(p, os.path.getsize(p))
