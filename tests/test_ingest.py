"""Scene ingest (fr_scene_load_obj, fr_texture_load) against the reference's
own loader: Scene::CreateScene with tinyobjloader 0.9.22 and stb_image 2.12,
run on the hand-made scene and images of tests/golden/ingest/ by
tests/golden/make_ingest_fixture.py.  Host code only, no GPU."""
import os
import struct
import sys
import zlib

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, GOLDEN)
import make_ingest_fixture as fx  # noqa: E402

INGEST = os.path.join(GOLDEN, 'ingest')
MESH = os.path.join(INGEST, 'meshData')


@pytest.fixture(scope='module')
def ref():
    return dict(np.load(os.path.join(GOLDEN, 'ingest_ref.npz')))


def material_table():
    """materials.txt as the harness's plug-in reads it (names not listed keep
    the default diffuse, non-SPPM surface)."""
    table = {}
    for line in open(os.path.join(INGEST, 'materials.txt')):
        n, t, sp, op, ix, r, e, rf = line.split()
        table[n] = dict(type=int(t), sppm=int(sp), opaque=int(op), index=float(ix), roughness=float(r),
                        extinction=float(e), reflectance=float(rf))
    return table


def image_names(ref):
    return sorted(k[4:] for k in ref if k.startswith('tex_'))


def test_textures_match_the_reference_loader(ref):
    """LoadTextureFromFile (stbi_load + the channel copy) of every fixture
    image: the same channel count and the same texels (c / 255.0f)."""
    from frsppm import abi
    names = image_names(ref)
    assert len(names) == 24
    for name in names:
        rgba, channels = abi.load_texture(os.path.join(MESH, name + '.png'))
        assert channels == int(ref['chan_' + name][0]), name
        np.testing.assert_array_equal(rgba.astype(np.float32) / np.float32(255.0), ref['tex_' + name], err_msg=name)


def test_obj_scene_matches_create_scene(ref):
    """Facets (positions, normals, UVs, attribute ids) bit for bit, the
    attribute table (Kd, Ke, the plug-in's surface parameters) and the
    texture bound to each attribute's albedo, roughness and normal map."""
    from frsppm import abi
    sc = abi.load_obj_scene(os.path.join(MESH, 'scene.obj'), asset_dir=MESH + '//', materials=material_table())
    np.testing.assert_array_equal(sc['pos'], ref['facet_pos'])
    np.testing.assert_array_equal(sc['nrm'], ref['facet_nrm'])
    np.testing.assert_array_equal(sc['uv'], ref['facet_uv'])
    np.testing.assert_array_equal(sc['mat'], ref['facet_attr'])
    m = sc['materials']
    assert [x['name'] for x in m] == ['white', 'red', 'blue', 'light', 'unusedmtl', 'white', '']
    np.testing.assert_array_equal(ref['attr_ids'], np.arange(len(m)))
    np.testing.assert_array_equal(np.array([x['albedo'] for x in m], np.float32), ref['attr_albedo'])
    np.testing.assert_array_equal(np.array([x['emission'] for x in m], np.float32), ref['attr_radiance'])
    params = np.array([[x['index'], x['roughness'], x['extinction'], x['reflectance'], x['sppm'], x['opaque']]
                       for x in m], np.float32)
    np.testing.assert_array_equal(params, ref['attr_params'])
    for k, x in enumerate(m):
        for slot, key in enumerate(('tex_albedo', 'tex_roughness', 'tex_bump')):
            fname = str(ref['attr_textures'][k][slot])
            if fname == '':
                assert x[key] == -1, (k, key)
            else:
                want, _ = abi.load_texture(os.path.join(MESH, os.path.basename(fname)))
                np.testing.assert_array_equal(sc['textures'][x[key]], want)
    assert len(sc['textures']) == 5  # one per file, shared by the materials naming it
    assert sc['ibl'] is None
    # The fixture's quirks as the reference has them.
    assert (sc['mat'] == -1).sum() == 2       # faces after "usemtl nosuch"
    assert np.isnan(sc['nrm']).sum() == 0


def test_default_material_plugin_keeps_the_attribute_defaults(ref):
    """No plug-in: every material is a diffuse surface that is not an SPPM
    surface, with SURFACE_PARAM()'s values and the MTL's Kd / Ke."""
    from frsppm import abi
    sc = abi.load_obj_scene(os.path.join(MESH, 'scene.obj'), asset_dir=MESH + '//')
    for x, kd, ke in zip(sc['materials'], ref['attr_albedo'], ref['attr_radiance']):
        assert (x['type'], x['sppm'], x['opaque']) == (0, False, True)
        assert (x['index'], x['roughness'], x['extinction'], x['reflectance']) == (1.0, 1.0, 1.0, 1.0)
        np.testing.assert_array_equal(np.float32(x['albedo']), kd)
        np.testing.assert_array_equal(np.float32(x['emission']), ke)


def _expected_rgba(px, ctype, depth, palette=None, trns=None):
    """What stbi_load + LoadTextureFromFile give for samples px (H, W, spp)
    when every row is decoded as the PNG specification says."""
    h, w, spp = px.shape
    out = np.zeros((h, w, 4), np.uint8)
    out[..., 3] = 255
    if ctype == 3:
        pal = np.full((256, 4), 255, np.int64)
        pal[:len(palette), :3] = palette
        if trns is not None:
            pal[:len(trns), 3] = list(trns)
        n = 4 if trns is not None else 3
        out[..., :n] = pal[px[..., 0]][..., :n]
        return out
    scale = {1: 255, 2: 85, 4: 17, 8: 1}[depth]
    out[..., :spp] = px * scale
    return out


@pytest.mark.parametrize('depth', [1, 2, 4])
@pytest.mark.parametrize('ctype', [0, 3])
@pytest.mark.parametrize('interlace', [0, 1])
def test_low_bit_depth_rows_with_every_filter(tmp_path, depth, ctype, interlace):
    """1/2/4-bit grey and palette images whose rows use all five filters
    decode to their samples (the reference's stb_image 2.12 reads the prior
    row of such images from unwritten memory for the Up, Average and Paeth
    filters, so they are checked against the encoded samples instead)."""
    from frsppm import abi
    rng = np.random.default_rng(depth * 10 + ctype + 100 * interlace)
    px = rng.integers(0, 1 << depth, size=(13, 11, 1))
    palette = rng.integers(0, 256, size=(1 << depth, 3)) if ctype == 3 else None
    p = tmp_path / 'low.png'
    p.write_bytes(fx.png_bytes(px, ctype, depth, palette=palette, interlace=interlace, filters=(0, 1, 2, 3, 4)))
    rgba, c = abi.load_texture(str(p))
    assert c == (3 if ctype == 3 else 1)
    np.testing.assert_array_equal(rgba, _expected_rgba(px, ctype, depth, palette))


def test_generated_scenes_round_trip_through_obj(tmp_path):
    """The OBJ/MTL/PNG files the scene generators write for the reference
    harness load back to the generators' own arrays, bit for bit (so the
    golden fixtures, made by the reference from those files, describe the
    scene the renderer gets either way)."""
    from frsppm import abi, objio, scenes
    for name, sc in [('cornell', scenes.cornell_box(width=32, height=32)), ('mixed_ibl', scenes.small_mixed(ibl=True)),
                     ('demo', scenes.demo_materials())]:
        d = str(tmp_path / name)
        objio.write_scene(sc, d)
        table = {m['name']: dict(type=m['type'], sppm=m['sppm'], opaque=m['opaque'], index=m['index'],
                                 roughness=m['roughness'], extinction=m['extinction'], reflectance=m['reflectance'])
                 for m in sc['materials']}
        md = os.path.join(d, 'meshData')
        env = os.path.join(md, 'ibl.png') if sc.get('ibl') is not None else None
        got = abi.load_obj_scene(os.path.join(md, 'scene.obj'), asset_dir=md + '//', environment=env,
                                 materials=table)
        for k in ('pos', 'nrm', 'uv'):
            np.testing.assert_array_equal(got[k], np.asarray(sc[k], np.float32), err_msg=name + ' ' + k)
        np.testing.assert_array_equal(got['mat'], sc['mat'])
        assert len(got['materials']) == len(sc['materials'])
        for a, b in zip(got['materials'], sc['materials']):
            assert a['name'] == b['name'] and a['type'] == b['type'] and a['sppm'] == bool(b['sppm'])
            np.testing.assert_array_equal(np.float32(a['albedo']), np.float32(b['albedo']))
            np.testing.assert_array_equal(np.float32(a['emission']), np.float32(b['emission']))
            for key in ('tex_albedo', 'tex_roughness', 'tex_bump'):
                if b[key] < 0:
                    assert a[key] == -1
                else:
                    np.testing.assert_array_equal(got['textures'][a[key]], sc['textures'][b[key]])
        if env:
            np.testing.assert_array_equal(got['ibl'], sc['ibl'])


def _write(path, text):
    with open(path, 'w') as f:
        f.write(text)
    return str(path)


def test_load_errors(tmp_path):
    """Files that cannot be read, faces naming vertices that do not exist and
    shapes mixing vertices with and without normals (which the reference
    reads past the end of its arrays) fail with FR_ERR_IO; a failing material
    plug-in fails the load."""
    from frsppm import abi
    with pytest.raises(RuntimeError, match=r'\(5\)'):
        abi.load_obj_scene(str(tmp_path / 'missing.obj'))
    bad = _write(tmp_path / 'bad.obj', 'v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n')
    with pytest.raises(RuntimeError, match='vertex 4 of 3'):
        abi.load_obj_scene(bad)
    mixed = _write(tmp_path / 'mixed.obj', 'v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1 2 3\nf 1//1 2//1 3//1\nf 3 2 1\n')
    with pytest.raises(RuntimeError, match='normals'):
        abi.load_obj_scene(mixed)
    ok = _write(tmp_path / 'ok.obj', 'mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nusemtl a\nf 1 2 3\n')
    _write(tmp_path / 'm.mtl', 'newmtl a\nKd 1 1 1\n')

    def boom(name, fields):
        raise ValueError('plug-in says no to ' + name)
    with pytest.raises(ValueError, match='no to a'):
        abi.load_obj_scene(ok, asset_dir=str(tmp_path) + '/', materials=boom)
    sc = abi.load_obj_scene(ok, asset_dir=str(tmp_path) + '/')
    assert sc['mat'].tolist() == [0] and sc['materials'][0]['name'] == 'a'
    # Without its MTL (asset_dir elsewhere) the loader still adds one default
    # material named "", and usemtl a names nothing: material -1.
    sc = abi.load_obj_scene(ok, asset_dir=str(tmp_path / 'nowhere') + '/')
    assert [m['name'] for m in sc['materials']] == [''] and sc['mat'].tolist() == [-1]
    # fr_create rejects material -1 before touching the device.
    from frsppm import scenes
    sc['camera'] = scenes.cornell_box(width=8, height=8)['camera']
    with pytest.raises(RuntimeError, match='material id -1'):
        abi.Renderer(sc, 1000)


def test_texture_errors(tmp_path):
    """Not a PNG, a truncated file, a corrupt deflate stream, a palette index
    past the palette, an unknown critical chunk: FR_ERR_IO."""
    from frsppm import abi
    good = fx.png_bytes(np.zeros((4, 4, 3), np.int64), 2, 8)
    cases = {
        'jpeg.png': b'\xff\xd8\xff\xe0' + b'\x00' * 32,
        'truncated.png': good[:len(good) // 2],
        'badzlib.png': good.replace(zlib.compress(bytes(4 * 13), 9), b'\x78\x9c\xff\xff\xff\xff'),
        'palette.png': fx.png_bytes(np.full((2, 2, 1), 7), 3, 8, palette=[[1, 2, 3]] * 4),
    }
    ihdr_end = 8 + 25
    crit = struct.pack('>I', 1) + b'ABCD' + b'\x00' + struct.pack('>I', zlib.crc32(b'ABCD\x00'))
    cases['critical.png'] = good[:ihdr_end] + crit + good[ihdr_end:]
    for name, data in cases.items():
        p = tmp_path / name
        p.write_bytes(data)
        with pytest.raises(RuntimeError, match=r'\(5\)'):
            abi.load_texture(str(p))
    # An ancillary chunk of unknown type is skipped.
    anc = good[:ihdr_end] + struct.pack('>I', 1) + b'abCD' + b'\x00' + struct.pack('>I', 0) + good[ihdr_end:]
    (tmp_path / 'anc.png').write_bytes(anc)
    rgba, c = abi.load_texture(str(tmp_path / 'anc.png'))
    assert c == 3 and rgba.shape == (4, 4, 4) and (rgba[..., 3] == 255).all()


def test_large_dynamic_stream_round_trip(tmp_path):
    """A 512 x 384 RGBA image at zlib level 9 (dynamic blocks, long matches,
    every distance code) and the library's own PNG writer (stored blocks)."""
    from frsppm import abi
    rng = np.random.default_rng(7)
    base = rng.integers(0, 256, size=(24, 40, 4))
    img = np.tile(base, (16, 13, 1))[:384, :512]
    img[::7, ::5] = rng.integers(0, 256, size=img[::7, ::5].shape)
    p = tmp_path / 'big.png'
    p.write_bytes(fx.png_bytes(img, 6, 8, filters=(0, 1, 2, 3, 4)))
    rgba, c = abi.load_texture(str(p))
    assert c == 4
    np.testing.assert_array_equal(rgba, img.astype(np.uint8))
    lib = abi.load()
    q = tmp_path / 'own.png'
    src = np.ascontiguousarray(img.astype(np.uint8))
    assert lib.fr_write_png(os.fsencode(str(q)), 512, 384, src.ctypes.data) == 0
    np.testing.assert_array_equal(abi.load_texture(str(q))[0], src)
