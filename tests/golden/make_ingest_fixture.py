"""Make the scene-ingest fixture: a hand-made OBJ/MTL scene and a set of PNG
images under tests/golden/ingest/, and what the reference's own loader makes
of them (oracle/_ref/frref, built from the reference sources) in
tests/golden/ingest_ref.npz.

    python tests/golden/make_ingest_fixture.py

The scene exercises what Scene::CreateScene and its OBJ loader
(tinyobjloader 0.9.22) do with: numbers in exponent form, with a leading '+',
or not numbers at all ('.5'); polygons; negative (relative) indices; v, v/vt,
v//vn and v/vt/vn corners; shapes with and without normals or texcoords;
"g" and "o" shape breaks, including the faces a usemtl flush right before a
"g" drops; an unknown usemtl name; a missing MTL library (one default
material named ""); a duplicated material name; map_Kd / map_d / map_bump /
bump textures, a shared one, a two-character name and a missing file;
CR LF, lone CR and a last line without an ending.  The PNG set covers every
colour type at every bit depth the format allows, tRNS on each kind, Adam7
interlacing, all five row filters, stored / fixed-Huffman / dynamic deflate
blocks, IDAT split over chunks and an ancillary chunk.  Images of 1, 2 or 4
bits per sample use only the None and Sub filters: for the Up, Average and
Paeth filters stb_image 2.12 takes the prior row from the start of the
previous row's output buffer while that row's bytes sit at its end
(stb_image.cpp:3547-3557), i.e. from memory not yet written, so the
reference's texture is undefined there (the library decodes those rows as
the PNG specification says; tests/test_ingest.py checks them against the
encoded samples).

ingest_ref.npz holds the harness's facets dump (facet_pos, facet_nrm,
facet_uv, facet_attr), the attribute table (attr_albedo, attr_radiance,
attr_params = index, roughness, extinction, reflectance, SPPM surface,
opaque; attr_textures = albedo, roughness and normal-map file names per
attribute), and per image tex_<name> (LoadTextureFromFile's float texels) and
chan_<name> (the channel count stbi_load reports).
"""
from __future__ import annotations

import os
import shutil
import struct
import subprocess
import sys
import tempfile
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
FRREF = os.path.join(REPO, 'oracle', '_ref', 'frref')
DIR = os.path.join(HERE, 'ingest')
MESH = os.path.join(DIR, 'meshData')


# -------------------------------------------------------------------- PNG encoder

def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def _pack_row(samples, depth):
    """One row of integer samples (already flattened over channels) as bytes."""
    if depth == 16:
        return b''.join(struct.pack('>H', int(s)) for s in samples)
    if depth == 8:
        return bytes(int(s) for s in samples)
    out, acc, nbits = bytearray(), 0, 0
    for s in samples:
        acc = (acc << depth) | int(s)
        nbits += depth
        if nbits == 8:
            out.append(acc)
            acc, nbits = 0, 0
    if nbits:
        out.append(acc << (8 - nbits))
    return bytes(out)


def _filter_rows(rows, bpp, filters):
    out, prev = bytearray(), bytes(len(rows[0])) if rows else b''
    for y, row in enumerate(rows):
        f = filters[y % len(filters)]
        enc = bytearray()
        for i, x in enumerate(row):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = (0, a, b, (a + b) >> 1, _paeth(a, b, c))[f]
            enc.append((x - pred) & 255)
        out.append(f)
        out += enc
        prev = row
    return bytes(out)


ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def png_bytes(px, ctype, depth, palette=None, trns=None, interlace=0, filters=(0,), level=9, strategy=None,
              idat_parts=1, ancillary=False):
    """px: (H, W, samples) integer samples at file depth (palette indices for
    colour type 3)."""
    h, w, spp = px.shape
    bpp = max(1, spp * depth // 8)
    if interlace:
        raw = b''
        for x0, y0, dx, dy in ADAM7:
            sub = px[y0::dy, x0::dx]
            if sub.shape[0] and sub.shape[1]:
                raw += _filter_rows([_pack_row(r.reshape(-1), depth) for r in sub], bpp, filters)
    else:
        raw = _filter_rows([_pack_row(r.reshape(-1), depth) for r in px], bpp, filters)
    if strategy is None:
        z = zlib.compress(raw, level)
    else:
        co = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
        z = co.compress(raw) + co.flush()

    def chunk(tag, data):
        return struct.pack('>I', len(data)) + tag + data + struct.pack('>I', zlib.crc32(tag + data) & 0xFFFFFFFF)

    out = b'\x89PNG\r\n\x1a\n' + chunk(b'IHDR', struct.pack('>IIBBBBB', w, h, depth, ctype, 0, 0, interlace))
    if ancillary:
        out += chunk(b'tEXt', b'Comment\x00ingest fixture')
    if palette is not None:
        out += chunk(b'PLTE', bytes(np.asarray(palette, np.uint8).reshape(-1)))
    if trns is not None:
        out += chunk(b'tRNS', trns)
    step = -(-len(z) // idat_parts)
    for k in range(idat_parts):
        out += chunk(b'IDAT', z[k * step:(k + 1) * step])
    return out + chunk(b'IEND', b'')


def images(rng):
    """name -> PNG bytes."""
    def u(shape, depth):
        return rng.integers(0, 1 << depth, size=shape)

    def key16(v):
        return struct.pack('>H', v)

    im = {}
    im['rgb8_filters'] = png_bytes(u((9, 13, 3), 8), 2, 8, filters=(0, 1, 2, 3, 4))
    im['rgba8_fixed'] = png_bytes(u((7, 11, 4), 8), 6, 8, filters=(4, 3), strategy=zlib.Z_FIXED)
    im['rgba8_stored'] = png_bytes(u((5, 9, 4), 8), 6, 8, filters=(1,), level=0)
    im['gray8'] = png_bytes(u((3, 16, 1), 8), 0, 8, filters=(1, 2, 3, 4))
    im['gray1'] = png_bytes(u((5, 17, 1), 1), 0, 1, filters=(0, 1))
    im['gray2'] = png_bytes(u((4, 9, 1), 2), 0, 2, filters=(1,))
    g4 = u((6, 10, 1), 4)
    g4[::2, ::3] = 9
    im['gray4_trns'] = png_bytes(g4, 0, 4, trns=key16(9), filters=(1, 0))
    im['graya8'] = png_bytes(u((7, 7, 2), 8), 4, 8, filters=(2, 1))
    im['graya16'] = png_bytes(u((4, 4, 2), 16), 4, 16)
    pal = rng.integers(0, 256, size=(200, 3))
    im['pal8'] = png_bytes(rng.integers(0, 200, size=(6, 12, 1)), 3, 8, palette=pal, filters=(0, 1))
    im['pal4_trns'] = png_bytes(u((9, 9, 1), 4), 3, 4, palette=rng.integers(0, 256, size=(16, 3)),
                                trns=bytes([0, 64, 128, 255, 7]), filters=(1,))
    im['pal2'] = png_bytes(u((3, 5, 1), 2), 3, 2, palette=rng.integers(0, 256, size=(4, 3)))
    im['pal1_trns'] = png_bytes(u((2, 19, 1), 1), 3, 1, palette=[[10, 20, 30], [200, 100, 50]], trns=bytes([33]))
    im['rgb16'] = png_bytes(u((5, 6, 3), 16), 2, 16, filters=(1, 4))
    im['rgba16'] = png_bytes(u((4, 5, 4), 16), 6, 16, filters=(2, 3))
    g16 = u((3, 7, 1), 16)
    g16[1, ::2] = 0x1234
    g16[2, 0] = 0x5534  # same low byte as the key: opaque at 16 bits
    im['gray16_trns'] = png_bytes(g16, 0, 16, trns=key16(0x1234))
    c8 = u((8, 8, 3), 8)
    c8[::3, ::2] = (17, 200, 3)
    c8[1, 1] = (17, 200, 4)
    im['rgb8_trns'] = png_bytes(c8, 2, 8, trns=key16(17) + key16(200) + key16(3), filters=(0, 4))
    g8 = u((4, 6, 1), 8)
    g8[:, 2] = 77
    im['gray8_trns'] = png_bytes(g8, 0, 8, trns=key16(77 + 256))  # the key's high byte is ignored at 8 bits
    im['rgba8_adam7'] = png_bytes(u((11, 13, 4), 8), 6, 8, interlace=1, filters=(0, 1, 2, 3, 4))
    im['gray1_adam7'] = png_bytes(u((5, 3, 1), 1), 0, 1, interlace=1, filters=(1,))
    im['pal4_adam7'] = png_bytes(u((7, 9, 1), 4), 3, 4, palette=rng.integers(0, 256, size=(16, 3)), interlace=1,
                                 filters=(0, 1))
    im['rgb8_multi_idat'] = png_bytes(u((17, 31, 3), 8), 2, 8, filters=(0, 1, 2), idat_parts=3, ancillary=True)
    tile = u((4, 6, 4), 8)
    im['rgba8_repeats'] = png_bytes(np.tile(tile, (12, 8, 1)), 6, 8, filters=(0, 2), level=9)
    im['rgba8_huffman_only'] = png_bytes(u((6, 6, 4), 3) * 30, 6, 8, strategy=zlib.Z_HUFFMAN_ONLY)
    return im


# ------------------------------------------------------------------- OBJ / MTL

MTL = """# ingest fixture materials
newmtl white
Kd 0.75 0.75 0.75
Ke 0 0 0
map_Kd rgb8_filters.png
map_d gray4_trns.png
map_bump pal8.png

newmtl red
Kd 0.75 0.25 2.5e-1
map_Kd rgb8_filters.png
bump graya8.png

newmtl blue
  Kd 0.25 0.25 0.75
map_Kd ab
map_d missing_texture.png

newmtl light
Kd 1 1 1
Ke 17 12 4
map_Kd rgba8_adam7.png

newmtl unusedmtl
Kd 0.1 0.2 0.3
Ka 1 1 1
illum 2

newmtl white
Kd 0.5 0.5 0.5
"""

# A 24 x 24 grid of quads (1152 triangles, not flat) in a shape of its own,
# and every other facet inside its extent: the
# reference's BVH build (Build3, bvh8.h:135-189, which CreateScene runs) writes
# through a triangle index as a node index when one of its 64 depth-2 nodes
# holds a single triangle (bvh8.h:181-189, 284-289), which corrupts memory and
# crashes small, flat or scattered scenes at random.
PAD_N = 24
PAD_LINES = ['o pad', 'usemtl white'] + [
    'v %g %g %g' % (x / PAD_N, y / PAD_N, 0.01 * ((x * 7 + y * 3) % 5) - 0.1)
    for y in range(PAD_N + 1) for x in range(PAD_N + 1)] + [
    'vn 0 0.6 0.8'] + [
    'f %d//4 %d//4 %d//4 %d//4' % (11 + y * (PAD_N + 1) + x, 12 + y * (PAD_N + 1) + x,
                                   12 + (y + 1) * (PAD_N + 1) + x, 11 + (y + 1) * (PAD_N + 1) + x)
    for y in range(PAD_N) for x in range(PAD_N)]

OBJ_LINES = [
    '# ingest fixture scene',
    'mtllib scene.mtl',
    'mtllib missing.mtl',
    'v 0 0 0',
    'v 1 0 0',
    'v 1 1 0',
    'v 0 1 0',
    'v 0.5 1.5e-1 2.25E-1',
    'v +0.125 .5 0.3',
    'v 1e-2 2.5e-1 -0.0',
    'v 0.7 0.8 0.09 1.0',
    '  v\t0.3333333333333333 0.1 0.2000000001',
    'v 1.25e-1 0.001 0.2',
    'vt 0 0',
    'vt 1 0',
    'vt 1 1',
    'vt 0 1',
    'vt 0.25 0.75',
    'vn 0 0 1',
    'vn 0 1 0',
    'vn 0.6 0.8 0',
    'o first',
    'usemtl white',
    'f 1 2 3',
    'f 1 3 4 ',
    'f 9 10 2',
    'g second group',
    'usemtl red',
    'f 1/1/1 2/2/1 3/3/1 4/4/1',
    'f -8/-5/-3 -7/-4/-2 -6/-3/-1',
    'usemtl white',
    'f 5/5/2 6/1/2 7/2/2 8/3/2 1/4/2',
    'f 1 2',
    'g lost',
    'usemtl red',
    'f 1/1/1 2/2/1 3/3/1',
    'usemtl light',
    'g kept',
    'usemtl light',
    'f 1/1 2/2 3/3',
    'f 3/3 4/4 1/1 2/5',
    'o tabs',
    'usemtl   blue  ',
    'f\t2//3\t3//3\t4//3',
    'usemtl nosuch',
    'f 2//3 4//3 1//3',
    's 1',
    'l 1 2',
    'vp 0.5',
    '',
    '   ',
    'g',
    'usemtl',
    'f 5//1 6//1 7//1',
    'usemtl blue',
    'f 8//2 9//2 10//2',
] + PAD_LINES + ['f 1//1 2//1 3//1']


def write_scene_files():
    if os.path.isdir(DIR):
        shutil.rmtree(DIR)
    os.makedirs(MESH)
    rng = np.random.default_rng(0x5EED1A5)
    for name, data in images(rng).items():
        with open(os.path.join(MESH, name + '.png'), 'wb') as f:
            f.write(data)
    with open(os.path.join(MESH, 'scene.mtl'), 'w', newline='') as f:
        f.write(MTL)
    # Line endings: mostly LF, some CR LF, one lone CR, none after the last line.
    text = ''
    for i, line in enumerate(OBJ_LINES):
        end = '' if i == len(OBJ_LINES) - 1 else ('\r\n' if i % 5 == 1 else ('\r' if i == 17 else '\n'))
        text += line + end
    with open(os.path.join(MESH, 'scene.obj'), 'w', newline='') as f:
        f.write(text)
    with open(os.path.join(DIR, 'materials.txt'), 'w') as f:
        # name type sppm opaque index roughness extinction reflectance (frsppm.objio.write_materials_table)
        f.write('white 0 1 1 1.5 0.5 1 1\n')
        f.write('red 2 1 1 1.5 0.2 2.5 0.9\n')
        f.write('blue 3 0 0 1.5 0.1 1 1\n')
        f.write('light 0 0 1 1 1 1 1\n')
        f.write('unusedmtl 1 0 1 1.2 0.3 1 1\n')
    with open(os.path.join(DIR, 'camera.txt'), 'w') as f:
        f.write('0 8 8\n0 0.5 3\n0 0.5 0\n60 1 1 1 0\n')


def run(args):
    r = subprocess.run([FRREF] + args, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('frref %s failed (%d): %s' % (' '.join(args), r.returncode, r.stderr))


def main():
    write_scene_files()
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        run([DIR, 'facets', tmp])
        for k in ('facet_pos', 'facet_nrm', 'facet_uv', 'facet_attr', 'attr_albedo', 'attr_radiance', 'attr_params'):
            out[k] = np.load(os.path.join(tmp, k + '.npy'))
        rows = [line.rstrip('\n').split('\t') for line in open(os.path.join(tmp, 'attr_textures.txt'))]
        out['attr_ids'] = np.array([int(r[0]) for r in rows], np.int32)
        out['attr_textures'] = np.array([r[1:] for r in rows])
        for fn in sorted(os.listdir(MESH)):
            if not fn.endswith('.png'):
                continue
            name = fn[:-4]
            d = os.path.join(tmp, name)
            os.makedirs(d)
            run([DIR, 'texture', os.path.join(MESH, fn), d])
            out['tex_' + name] = np.load(os.path.join(d, 'texels.npy'))
            out['chan_' + name] = np.load(os.path.join(d, 'channels.npy'))
    np.savez_compressed(os.path.join(HERE, 'ingest_ref.npz'), **out)
    print('facets', len(out['facet_attr']), 'attributes', len(out['attr_ids']),
          'images', sum(k.startswith('tex_') for k in out))


if __name__ == '__main__':
    sys.exit(main())
