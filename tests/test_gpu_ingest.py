"""A scene read from OBJ/MTL/PNG files by fr_scene_load_obj renders on the
GPU what the reference renders from the same files: the golden fixtures were
made by the reference's CreateScene + render on exactly the files
frsppm.objio writes.  Per-pixel photon counts N exact, the image within
1e-4 relative of the reference's and within float rounding (1e-5) of the
render of the generator's arrays."""
import os

import numpy as np
import pytest

from conftest import GOLDEN_SCENES, load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('name', ['cornell32', 'mixed48x32_ibl', 'demo48x32'])
def test_render_from_obj_matches_reference(tmp_path, name):
    from frsppm import abi, objio
    gold = load_golden(name)
    sc = GOLDEN_SCENES[name]()
    objio.write_scene(sc, str(tmp_path))
    table = {m['name']: dict(type=m['type'], sppm=m['sppm'], opaque=m['opaque'], index=m['index'],
                             roughness=m['roughness'], extinction=m['extinction'], reflectance=m['reflectance'])
             for m in sc['materials']}
    md = os.path.join(str(tmp_path), 'meshData')
    env = os.path.join(md, 'ibl.png') if sc.get('ibl') is not None else None
    loaded = abi.load_obj_scene(os.path.join(md, 'scene.obj'), asset_dir=md + '//', environment=env,
                                materials=table)
    loaded['camera'] = sc['camera']
    iters = int(gold['iters'])
    images = []
    for scene in (loaded, sc):
        with abi.Renderer(scene, int(gold['photons']), alpha=0.9, radius=0.015) as r:
            r.iterate(iters)
            images.append(r.resolve())
            st = r.read_state()
        np.testing.assert_array_equal(st['n'], gold['it%d_sp_n' % iters])
    ref = gold['image']
    err = np.abs(images[0] - ref).max() / np.abs(ref).max()
    assert err < 1e-4, err
    # A grid cell's photons are summed in the order its atomic counter gave
    # them slots, so two renders agree to float rounding.
    assert np.abs(images[0] - images[1]).max() <= 1e-5 * np.abs(images[1]).max()
