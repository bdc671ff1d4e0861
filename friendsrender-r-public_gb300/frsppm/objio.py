"""Scene file I/O: RGBA8 PNG, and OBJ/MTL in the layout the reference's
``Scene::CreateScene`` reads (SPPM/SPPM/Scene.cpp:13-77, tinyobjloader 0.9.22).

Floats are written with 9 significant digits, which round-trips float32
exactly through the loader's ``(float)atof`` (tiny_obj_loader.cpp:255-258).
Every facet corner gets its own ``v``/``vt``/``vn`` so facet ``f`` of the
arrays is face ``f`` of the file.  MTL keys follow the reference's mapping
(Scene.cpp:60-77): ``map_Kd`` albedo, ``map_d`` roughness, ``map_bump``
normal map; ``Kd`` albedo and ``Ke`` emission."""
from __future__ import annotations

import os
import struct
import zlib

import numpy as np


def write_png_rgba(path, img):
    """Write an (H, W, 4) uint8 array as an 8-bit RGBA PNG (filter 0 rows)."""
    img = np.ascontiguousarray(img, np.uint8)
    h, w, c = img.shape
    assert c == 4
    raw = b''.join(b'\x00' + img[y].tobytes() for y in range(h))

    def chunk(tag, data):
        body = tag + data
        return struct.pack('>I', len(data)) + body + struct.pack('>I', zlib.crc32(body) & 0xFFFFFFFF)

    png = b'\x89PNG\r\n\x1a\n' + chunk(b'IHDR', struct.pack('>IIBBBBB', w, h, 8, 6, 0, 0, 0))
    png += chunk(b'IDAT', zlib.compress(raw, 6)) + chunk(b'IEND', b'')
    with open(path, 'wb') as f:
        f.write(png)


def _f(x):
    return '%.9g' % float(np.float32(x))


def write_scene(scene, directory, name='scene'):
    """Write ``directory/meshData/{name}.obj``, ``{name}.mtl`` and ``tex{i}.png``;
    returns the OBJ path relative to ``directory`` (the reference resolves
    MTL and texture names against ``meshData//``, Scene.cpp:20-21)."""
    md = os.path.join(directory, 'meshData')
    os.makedirs(md, exist_ok=True)
    for i, tex in enumerate(scene['textures']):
        write_png_rgba(os.path.join(md, 'tex%d.png' % i), tex)
    if scene.get('ibl') is not None:  # environment map (the reference's IBL texture)
        write_png_rgba(os.path.join(md, 'ibl.png'), scene['ibl'])
    with open(os.path.join(md, name + '.mtl'), 'w') as f:
        for m in scene['materials']:
            f.write('newmtl %s\n' % m['name'])
            f.write('Kd %s %s %s\n' % tuple(_f(x) for x in m['albedo']))
            f.write('Ke %s %s %s\n' % tuple(_f(x) for x in m['emission']))
            if m['tex_albedo'] >= 0:
                f.write('map_Kd tex%d.png\n' % m['tex_albedo'])
            if m['tex_roughness'] >= 0:
                f.write('map_d tex%d.png\n' % m['tex_roughness'])
            if m['tex_bump'] >= 0:
                f.write('map_bump tex%d.png\n' % m['tex_bump'])
            f.write('\n')
    pos, nrm, uv, mat = scene['pos'], scene['nrm'], scene['uv'], scene['mat']
    lines = ['mtllib %s.mtl\n' % name, 'o scene\n']
    current = None
    for t in range(len(pos)):
        for k in range(3):
            lines.append('v %s %s %s\n' % tuple(_f(x) for x in pos[t, k]))
            lines.append('vt %s %s\n' % tuple(_f(x) for x in uv[t, k]))
            lines.append('vn %s %s %s\n' % tuple(_f(x) for x in nrm[t, k]))
        if mat[t] != current:
            current = int(mat[t])
            lines.append('usemtl %s\n' % scene['materials'][current]['name'])
        b = 3 * t + 1
        lines.append('f %d/%d/%d %d/%d/%d %d/%d/%d\n' % (b, b, b, b + 1, b + 1, b + 1, b + 2, b + 2, b + 2))
    with open(os.path.join(md, name + '.obj'), 'w') as f:
        f.writelines(lines)
    return os.path.join('meshData', name + '.obj')


def write_materials_table(scene, path):
    """Material table for the reference harness's SceneMaterialManager plug-in:
    one line per material: name type sppm opaque index roughness extinction reflectance."""
    with open(path, 'w') as f:
        for m in scene['materials']:
            f.write('%s %d %d %d %s %s %s %s\n' % (
                m['name'], m['type'], int(m['sppm']), int(m['opaque']), _f(m['index']),
                _f(m['roughness']), _f(m['extinction']), _f(m['reflectance'])))


def write_camera(scene, path):
    """Camera parameters for the reference harness (iCamera ctor, Camera.h:132-151)."""
    c = scene['camera']
    with open(path, 'w') as f:
        f.write('%d %d %d\n' % (c['type'], c['width'], c['height']))
        f.write('%s %s %s\n' % tuple(_f(x) for x in c['pos']))
        f.write('%s %s %s\n' % tuple(_f(x) for x in c['target']))
        f.write('%s %s %s %s %s\n' % tuple(_f(x) for x in (c['fov'], c['focal'], c['dist'], c['aspect'], c['lens'])))
