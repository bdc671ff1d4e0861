"""Seeded synthetic SPPM scenes as flat numpy arrays.

A scene is a dict of arrays in exactly the per-facet form the reference builds
in ``Scene::CreateScene`` (SPPM/SPPM/Scene.cpp:182-236): facet ``f`` has three
corner positions, three corner normals and three corner UVs, plus a material
(attribute) id.  Facet order is the OBJ face order, so the same arrays can be
written as OBJ/MTL/PNG for the reference loader (``objio.write_scene``) and
handed unchanged to the C-ABI (``fr_scene_desc``).

Material records mirror the ``SURFACE_PARAM`` fields the reference's
``SceneMaterialManager`` plug-in sets (SPPM/SPPM/material.h:35-90,
SPPM/SPPM/main.cpp:14-114); ``type`` selects the ``Surface`` subclass:

    0 DiffuseSurface   (material.h:163-177)
    1 MetalSurface     (material.h:396-425)   perfect mirror
    2 Roughconductor   (material.h:222-278)   GGX conductor
    3 GGXGlass         (material.h:280-394)   GGX dielectric

All randomness comes from ``numpy.random.Generator(PCG64(seed))``.
"""
from __future__ import annotations

import math

import numpy as np

DIFFUSE, METAL, GGX_CONDUCTOR, GGX_DIELECTRIC = 0, 1, 2, 3
# The demo's further surfaces (material.h:427-766, used by main.cpp:14-114).
BIMETAL, GLASS, GLOSS_TRANSMIT, DIFFUSE_TRANSMIT = 4, 5, 6, 7
PINHOLE, THINLENS = 0, 1

CONFIG_SEED_BASE = 0x5EED0000


def material(name, mtype, albedo=(0.75, 0.75, 0.75), emission=(0.0, 0.0, 0.0),
             roughness=1.0, index=1.0, extinction=1.0, reflectance=1.0,
             opaque=True, sppm=True, tex_albedo=-1, tex_roughness=-1, tex_bump=-1):
    """One material record.  Defaults are the reference's SURFACE_PARAM()
    defaults (material.h:76-89) except ``isSPPMSurface``, which the reference's
    default manager leaves false (no hitpoints at all); scenes set it."""
    return dict(name=name, type=int(mtype), albedo=tuple(float(x) for x in albedo),
                emission=tuple(float(x) for x in emission), roughness=float(roughness),
                index=float(index), extinction=float(extinction),
                reflectance=float(reflectance), opaque=bool(opaque), sppm=bool(sppm),
                tex_albedo=int(tex_albedo), tex_roughness=int(tex_roughness),
                tex_bump=int(tex_bump))


class _Builder:
    def __init__(self):
        self.pos, self.nrm, self.uv, self.mat = [], [], [], []

    def tris(self, p, n, uv, mat_id):
        p = np.asarray(p, np.float32).reshape(-1, 3, 3)
        n = np.asarray(n, np.float32).reshape(-1, 3, 3)
        uv = np.asarray(uv, np.float32).reshape(-1, 3, 2)
        self.pos.append(p)
        self.nrm.append(n)
        self.uv.append(uv)
        self.mat.append(np.full(len(p), mat_id, np.int32))

    def quad(self, a, b, c, d, normal, mat_id, uvs=((0, 0), (1, 0), (1, 1), (0, 1))):
        """Quad a-b-c-d as triangles (a,b,c) and (a,c,d), flat normal."""
        a, b, c, d = (np.asarray(x, np.float32) for x in (a, b, c, d))
        nrm = np.asarray(normal, np.float32)
        u = [np.asarray(x, np.float32) for x in uvs]
        self.tris([[a, b, c], [a, c, d]], [[nrm] * 3, [nrm] * 3],
                  [[u[0], u[1], u[2]], [u[0], u[2], u[3]]], mat_id)

    def build(self):
        return dict(pos=np.concatenate(self.pos).astype(np.float32),
                    nrm=np.concatenate(self.nrm).astype(np.float32),
                    uv=np.concatenate(self.uv).astype(np.float32),
                    mat=np.concatenate(self.mat).astype(np.int32))


def _rot_y(deg):
    t = math.radians(deg)
    c, s = math.cos(t), math.sin(t)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], np.float64)


def _box(b, center, size, rot_deg, mat_id):
    """Axis-aligned box rotated about y: 12 triangles, outward flat normals."""
    R = _rot_y(rot_deg)
    hx, hy, hz = (s * 0.5 for s in size)
    corners = np.array([[x, y, z] for x in (-hx, hx) for y in (-hy, hy) for z in (-hz, hz)])
    corners = corners @ R.T + np.asarray(center)
    faces = [  # (corner ids ccw seen from outside, outward local normal)
        ((0, 1, 3, 2), (-1, 0, 0)), ((4, 6, 7, 5), (1, 0, 0)),
        ((0, 4, 5, 1), (0, -1, 0)), ((2, 3, 7, 6), (0, 1, 0)),
        ((0, 2, 6, 4), (0, 0, -1)), ((1, 5, 7, 3), (0, 0, 1)),
    ]
    for (i0, i1, i2, i3), n in faces:
        nw = R @ np.asarray(n, np.float64)
        b.quad(corners[i0], corners[i1], corners[i2], corners[i3], nw, mat_id)


def _camera(ctype, width, height, pos, target, fov, focal=1.0, dist=1.0,
            lens=0.0):
    return dict(type=int(ctype), width=int(width), height=int(height),
                pos=tuple(float(x) for x in pos), target=tuple(float(x) for x in target),
                fov=float(fov), focal=float(focal), dist=float(dist),
                aspect=float(width) / float(height), lens=float(lens))


def value_noise(rng, size, cells, channels=1):
    """Seeded value noise: a coarse random grid, bilinearly upsampled (float64 in [0,1])."""
    grid = rng.random((cells + 1, cells + 1, channels))
    t = np.linspace(0.0, cells, size, endpoint=False)
    i0 = np.floor(t).astype(int)
    f = t - i0
    g00 = grid[i0][:, i0]
    g10 = grid[i0 + 1][:, i0]
    g01 = grid[i0][:, i0 + 1]
    g11 = grid[i0 + 1][:, i0 + 1]
    fy = f[:, None, None]
    fx = f[None, :, None]
    return (g00 * (1 - fy) * (1 - fx) + g10 * fy * (1 - fx) + g01 * (1 - fy) * fx + g11 * fy * fx)


def noise_texture(rng, size, kind):
    """RGBA8 seeded texture.  ``kind``: 'albedo' | 'roughness' | 'normal' | 'emission'.
    Alpha is 255 (opaque) so no surface takes the reference's translucency
    pass-through (SPPM.cpp:138-142) unless a scene asks for it explicitly."""
    n = value_noise(rng, size, max(4, size // 64), 3) * 0.6 + value_noise(rng, size, max(8, size // 16), 3) * 0.4
    if kind == 'albedo':
        rgb = 0.15 + 0.8 * n
    elif kind == 'roughness':
        rgb = np.repeat(n[..., :1], 3, axis=2) * 0.9 + 0.1
    elif kind == 'normal':
        rgb = np.empty_like(n)
        rgb[..., 0] = 0.5 + 0.25 * (n[..., 0] - 0.5)
        rgb[..., 1] = 0.5 + 0.25 * (n[..., 1] - 0.5)
        rgb[..., 2] = 0.9 + 0.1 * n[..., 2]
    elif kind == 'emission':
        rgb = 0.3 + 0.7 * n
    else:
        raise ValueError(kind)
    out = np.empty((size, size, 4), np.uint8)
    out[..., :3] = np.clip(np.round(rgb * 255.0), 0, 255).astype(np.uint8)
    out[..., 3] = 255
    return out


def sky_texture(rng, width=128, height=64):
    """RGBA8 equirectangular environment map for the reference's IBL (SPHERE
    mapping: u around y, v = acos(y) / pi from the top): a seeded sky, bright
    near the top, with value noise."""
    v = (np.arange(height) + 0.5)[:, None] / height
    n = value_noise(rng, max(width, height), 8, 3)[:height, :width]
    base = np.clip(1.0 - v, 0.0, 1.0)[..., None] * np.array([0.55, 0.7, 1.0]) + 0.15
    rgb = np.clip(base * (0.75 + 0.5 * n), 0.0, 1.0)
    out = np.empty((height, width, 4), np.uint8)
    out[..., :3] = np.round(rgb * 255.0).astype(np.uint8)
    out[..., 3] = 255
    return out


def with_sky(scene, seed):
    """The scene lit also by a seeded environment map (sky_texture)."""
    scene['ibl'] = sky_texture(np.random.Generator(np.random.PCG64(seed)))
    return scene


def cornell_box(seed=CONFIG_SEED_BASE + 0, width=256, height=256, light_rgb=(17.0, 12.0, 4.0)):
    """Procedural Cornell box: unit cube with 5 diffuse walls, a diffuse box and
    a GGX-conductor box (roughness 0.2) rotated by U(0,30) degrees, and a
    0.25x0.25 ceiling quad light.  34 scene triangles + 2 light triangles.

    The light sits 1e-3 below the ceiling so no camera or photon ray meets two
    coplanar triangles at the same distance (the reference resolves such ties
    by BVH visit order, bvh8.h:591)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    mats = [
        material('white', DIFFUSE, (0.75, 0.75, 0.75)),
        material('red', DIFFUSE, (0.75, 0.25, 0.25)),
        material('green', DIFFUSE, (0.25, 0.75, 0.25)),
        material('boxdiffuse', DIFFUSE, (0.75, 0.75, 0.75)),
        material('boxconductor', GGX_CONDUCTOR, (0.9, 0.85, 0.8), roughness=0.2,
                 index=1.1978, extinction=7.0488),
        material('light', DIFFUSE, (1.0, 1.0, 1.0), emission=light_rgb),
    ]
    b = _Builder()
    b.quad((0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0), (0, 1, 0), 0)        # floor
    b.quad((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1), (0, -1, 0), 0)       # ceiling
    b.quad((0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1), (0, 0, -1), 0)       # back
    b.quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1), (1, 0, 0), 1)        # left (red)
    b.quad((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0), (-1, 0, 0), 2)       # right (green)
    r1, r2 = rng.uniform(0.0, 30.0, 2)
    # Boxes float 1e-3 above the floor for the same reason (no coplanar faces).
    _box(b, (0.33, 0.301, 0.62), (0.27, 0.6, 0.27), r1, 3)
    _box(b, (0.68, 0.151, 0.35), (0.27, 0.3, 0.27), -r2, 4)
    y = 1.0 - 1e-3
    b.quad((0.375, y, 0.375), (0.625, y, 0.375), (0.625, y, 0.625), (0.375, y, 0.625),
           (0, -1, 0), 5)
    scene = b.build()
    scene.update(materials=mats, textures=[],
                 camera=_camera(PINHOLE, width, height, (0.5, 0.5, -1.35), (0.5, 0.5, 0.5), 38.0))
    return scene


def uv_sphere(b, center, radius, mat_id, n_lat=34, n_lon=36, uv_scale=1.0):
    """UV sphere with smooth normals: 2*n_lon cap triangles + 2*n_lon*(n_lat-2) band triangles."""
    c = np.asarray(center, np.float64)
    th = np.linspace(0.0, math.pi, n_lat + 1)
    ph = np.linspace(0.0, 2.0 * math.pi, n_lon + 1)
    st, ct = np.sin(th), np.cos(th)
    dirs = np.stack([st[:, None] * np.cos(ph)[None, :], np.repeat(ct[:, None], n_lon + 1, 1),
                     st[:, None] * np.sin(ph)[None, :]], axis=-1)
    pts = c + radius * dirs
    uvs = np.stack(np.meshgrid(ph / (2 * math.pi), th / math.pi), -1) * uv_scale
    P, N, U = [], [], []
    for i in range(n_lat):
        for j in range(n_lon):
            a, bb = (i, j), (i, j + 1)
            cc, d = (i + 1, j + 1), (i + 1, j)
            if i != 0:
                P.append([pts[a], pts[bb], pts[cc]]); N.append([dirs[a], dirs[bb], dirs[cc]])
                U.append([uvs[a], uvs[bb], uvs[cc]])
            if i != n_lat - 1:
                P.append([pts[a], pts[cc], pts[d]]); N.append([dirs[a], dirs[cc], dirs[d]])
                U.append([uvs[a], uvs[cc], uvs[d]])
    b.tris(P, N, U, mat_id)


def height_field(b, rng, n, x0, x1, z0, z1, amp, mat_id, uv_scale=4.0):
    """n x n vertex grid of seeded value noise: 2*(n-1)^2 triangles, smooth normals."""
    h = value_noise(rng, n, max(4, n // 32), 1)[..., 0] * amp
    xs = np.linspace(x0, x1, n)
    zs = np.linspace(z0, z1, n)
    X, Z = np.meshgrid(xs, zs, indexing='xy')
    P = np.stack([X, h, Z], -1)
    gx = np.gradient(h, xs, axis=1)
    gz = np.gradient(h, zs, axis=0)
    Nn = np.stack([-gx, np.ones_like(h), -gz], -1)
    Nn /= np.linalg.norm(Nn, axis=-1, keepdims=True)
    U = np.stack(np.meshgrid(np.linspace(0, uv_scale, n), np.linspace(0, uv_scale, n), indexing='xy'), -1)
    i, j = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing='ij')
    i, j = i.ravel(), j.ravel()
    a, bb, cc, d = (i, j), (i, j + 1), (i + 1, j + 1), (i + 1, j)
    def tri(p, q, r):
        return (np.stack([P[p], P[q], P[r]], 1), np.stack([Nn[p], Nn[q], Nn[r]], 1),
                np.stack([U[p], U[q], U[r]], 1))
    t1 = tri(a, d, cc)
    t2 = tri(a, cc, bb)
    inter = lambda k: np.stack([t1[k], t2[k]], 1).reshape(-1, 3, t1[k].shape[-1])
    b.tris(inter(0), inter(1), inter(2), mat_id)


def mixed_materials(seed=CONFIG_SEED_BASE + 1, width=1280, height=720, n_spheres=200,
                    field_n=512, tex_size=1024, light_tex=512, n_lat=34, n_lon=36,
                    aperture=0.02, extent=4.0):
    """Mixed-materials scene: ``n_spheres`` UV spheres (radius U(0.05,0.3)) over a
    ``field_n``^2 height field of seeded value noise.  Materials split equally
    across diffuse, specular, GGX conductor and GGX dielectric (IOR 1.5),
    roughness U(0.05,0.5).  The field carries albedo/roughness/normal textures
    (``tex_size``^2 RGBA8), the area light a ``light_tex``^2 textured emission,
    and the camera is a thin lens with aperture ``aperture``.
    With the defaults: 997,444 triangles at 1280x720."""
    rng = np.random.Generator(np.random.PCG64(seed))
    textures = [noise_texture(rng, tex_size, 'albedo'), noise_texture(rng, tex_size, 'roughness'),
                noise_texture(rng, tex_size, 'normal'), noise_texture(rng, light_tex, 'emission')]
    mats = [material('field', DIFFUSE, (0.7, 0.7, 0.7), tex_albedo=0, tex_roughness=1, tex_bump=2),
            material('light', DIFFUSE, (1, 1, 1), emission=(10.0, 9.0, 8.0), tex_albedo=3)]
    b = _Builder()
    ext = float(extent)
    k_s = ext / 4.0  # lengths below are for the 8x8 field and scale with it
    height_field(b, rng, field_n, -ext, ext, -ext, ext, 0.25 * k_s, 0)
    for k in range(n_spheres):
        mtype = k % 4
        rough = float(rng.uniform(0.05, 0.5))
        col = tuple(float(x) for x in rng.uniform(0.3, 0.95, 3))
        name = 's%03d' % k
        if mtype == DIFFUSE:
            m = material(name, DIFFUSE, col)
        elif mtype == METAL:
            m = material(name, METAL, col, sppm=False)
        elif mtype == GGX_CONDUCTOR:
            m = material(name, GGX_CONDUCTOR, col, roughness=rough, index=1.1978, extinction=7.0488)
        else:
            m = material(name, GGX_DIELECTRIC, (0.98, 0.98, 0.98), roughness=rough, index=1.5,
                         opaque=False, sppm=False)
        mats.append(m)
        r = float(rng.uniform(0.05, 0.3)) * k_s
        cx, cz = rng.uniform(-ext * 0.85, ext * 0.85, 2)
        uv_sphere(b, (cx, 0.25 * k_s + r, cz), r, len(mats) - 1, n_lat, n_lon)
    ly, lh = 3.0 * k_s, 1.0 * k_s
    b.quad((-lh, ly, -lh), (lh, ly, -lh), (lh, ly, lh), (-lh, ly, lh), (0, -1, 0), 1)
    scene = b.build()
    scene.update(materials=mats, textures=textures,
                 camera=_camera(THINLENS, width, height, (0.0, 2.6 * k_s, -7.5 * k_s), (0.0, 0.2 * k_s, 0.0),
                                30.0, focal=0.9, dist=1.0, lens=aperture))
    return scene


def caustic_box(seed=CONFIG_SEED_BASE + 2, width=1024, height=1024, n_spheres=50, n_lat=40, n_lon=51,
                light_tex=256, slit=0.1):
    """Caustic scene: a 1x1 textured area light above a diffuse box whose only
    opening is a ``slit`` x ``slit`` hole in its top, so most photons of plain
    light sampling never enter.  Inside, ``n_spheres`` GGX-dielectric spheres
    (IOR 1.5, roughness 0.02) stand on the diffuse floor and focus the light
    that comes through the slit into caustics.  A pinhole camera inside the
    box looks at the floor (its image plane, where the reference's pinhole
    camera starts its rays, sits 0.01 behind the pinhole so that it is inside
    the box too).  With the defaults: 198,936 triangles, 1024^2."""
    rng = np.random.Generator(np.random.PCG64(seed))
    textures = [noise_texture(rng, light_tex, 'emission')]
    mats = [material('floor', DIFFUSE, (0.8, 0.8, 0.8)),
            material('walls', DIFFUSE, (0.7, 0.65, 0.6)),
            material('glass', GGX_DIELECTRIC, (0.98, 0.98, 0.98), roughness=0.02, index=1.5,
                     opaque=False, sppm=False),
            material('light', DIFFUSE, (1, 1, 1), emission=(40.0, 36.0, 32.0), tex_albedo=0)]
    b = _Builder()
    x0, x1, y1, h = -1.0, 1.0, 1.2, slit * 0.5
    b.quad((x0, 0, x0), (x0, 0, x1), (x1, 0, x1), (x1, 0, x0), (0, 1, 0), 0)            # floor
    b.quad((x0, 0, x0), (x0, y1, x0), (x0, y1, x1), (x0, 0, x1), (1, 0, 0), 1)          # walls
    b.quad((x1, 0, x0), (x1, 0, x1), (x1, y1, x1), (x1, y1, x0), (-1, 0, 0), 1)
    b.quad((x0, 0, x1), (x0, y1, x1), (x1, y1, x1), (x1, 0, x1), (0, 0, -1), 1)
    b.quad((x0, 0, x0), (x1, 0, x0), (x1, y1, x0), (x0, y1, x0), (0, 0, 1), 1)
    # Top: a slab of thickness t with the slit at its centre (inner and outer
    # faces as four rectangles around the hole, and the hole's four sides), so
    # photons stopped on the outside lie farther than a gather radius from the
    # hitpoints inside.  The slab overhangs the walls (to +-1.5), so light from
    # the 1x1 light that passes the slab's edge travels outward and never lands
    # on the outer side of the (zero-thickness) walls, where interior
    # hitpoints would count it.
    t, o = 0.05, 1.5
    for y, ny in ((y1, -1), (y1 + t, 1)):
        for (a0, a1, c0, c1) in ((-o, -h, -o, o), (h, o, -o, o), (-h, h, -o, -h), (-h, h, h, o)):
            b.quad((a0, y, c0), (a1, y, c0), (a1, y, c1), (a0, y, c1), (0, ny, 0), 1)
    b.quad((-h, y1, -h), (-h, y1 + t, -h), (-h, y1 + t, h), (-h, y1, h), (1, 0, 0), 1)
    b.quad((h, y1, -h), (h, y1, h), (h, y1 + t, h), (h, y1 + t, -h), (-1, 0, 0), 1)
    b.quad((-h, y1, -h), (h, y1, -h), (h, y1 + t, -h), (-h, y1 + t, -h), (0, 0, 1), 1)
    b.quad((-h, y1, h), (-h, y1 + t, h), (h, y1 + t, h), (h, y1, h), (0, 0, -1), 1)
    placed = []
    while len(placed) < n_spheres:
        r = float(rng.uniform(0.05, 0.15))
        cx, cz = (float(v) for v in rng.uniform(-0.85, 0.85, 2))
        if all((cx - px) ** 2 + (cz - pz) ** 2 > (r + pr + 0.01) ** 2 for px, pz, pr in placed):
            placed.append((cx, cz, r))
    for cx, cz, r in placed:
        uv_sphere(b, (cx, r + 1e-3, cz), r, 2, n_lat, n_lon)
    ly = 1.6
    b.quad((-0.5, ly, -0.5), (0.5, ly, -0.5), (0.5, ly, 0.5), (-0.5, ly, 0.5), (0, -1, 0), 3)
    scene = b.build()
    scene.update(materials=mats, textures=textures,
                 camera=_camera(PINHOLE, width, height, (0.0, 0.95, -0.95), (0.0, 0.0, 0.15), 75.0, dist=0.01))
    return scene


def geodesic_sphere(freq):
    """Unit geodesic sphere: every face of an icosahedron split into freq^2
    triangles and projected to the sphere.  Returns unit directions (20*freq^2,
    3, 3), counter-clockwise seen from outside."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
             (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    n = int(freq)
    ii, jj = [], []
    for i in range(n):
        for j in range(n - i):
            ii.append((i, j, i + 1, j, i, j + 1))
            if i + j < n - 1:
                ii.append((i + 1, j, i + 1, j + 1, i, j + 1))
    idx = np.asarray(ii, np.float64).reshape(-1, 3, 2) / n  # (n^2, 3, [bary_b, bary_c])
    out = []
    for a, b, c in faces:
        A, Bv, Cv = v[a], v[b], v[c]
        P = A + idx[..., :1] * (Bv - A) + idx[..., 1:2] * (Cv - A)
        out.append(P / np.linalg.norm(P, axis=-1, keepdims=True))
    return np.concatenate(out)


def _displaced_sphere(rng, freq, amp, waves=12):
    """A geodesic sphere displaced radially by a seeded sum of plane waves
    h(d) = amp * sum_k a_k cos(f_k . d + p_k): positions, analytic normals
    and spherical UVs (each (tris, 3, k))."""
    d = geodesic_sphere(freq)
    f = rng.normal(size=(waves, 3)) * 3.0
    a = rng.uniform(0.3, 1.0, waves) / waves
    ph = rng.uniform(0.0, 2.0 * math.pi, waves)
    arg = d @ f.T + ph
    h = amp * (np.cos(arg) @ a)
    g = -amp * (np.sin(arg) * a) @ f                          # gradient of h
    gt = g - np.sum(g * d, axis=-1, keepdims=True) * d       # its tangential part
    r = 1.0 + h
    pos = d * r[..., None]
    nrm = d - gt / r[..., None]
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    uv = np.stack([np.arctan2(d[..., 2], d[..., 0]) / (2 * math.pi) + 0.5,
                   np.arccos(np.clip(d[..., 1], -1.0, 1.0)) / math.pi], -1)
    return pos, nrm, uv


def large_scene(seed=CONFIG_SEED_BASE + 4, width=3840, height=2160, instances=400, freq=50, tex_size=4096,
                light_tex=512, aperture=0.02, extent=10.0):
    """Large scene: ``instances`` copies of one seeded displaced geodesic sphere
    of 20*freq^2 triangles (50,000 with the default), each scaled, turned about
    y and placed on a textured ground quad, flattened into one triangle list
    (the boundary takes no instances).  16 materials cycle over the copies,
    four of each type (diffuse with the ground's textures, specular, GGX
    conductor, GGX dielectric IOR 1.5); the ground carries ``tex_size``^2 RGBA8
    albedo/roughness/normal textures; a ``light_tex``^2 textured area light;
    thin-lens camera (aperture ``aperture``).  With the defaults: 20,000,004
    triangles at 3840x2160."""
    rng = np.random.Generator(np.random.PCG64(seed))
    textures = [noise_texture(rng, tex_size, 'albedo'), noise_texture(rng, tex_size, 'roughness'),
                noise_texture(rng, tex_size, 'normal'), noise_texture(rng, light_tex, 'emission')]
    mats = [material('ground', DIFFUSE, (0.7, 0.7, 0.7), tex_albedo=0, tex_roughness=1, tex_bump=2),
            material('light', DIFFUSE, (1, 1, 1), emission=(30.0, 28.0, 25.0), tex_albedo=3)]
    for k in range(16):
        mtype = k % 4
        rough = float(rng.uniform(0.05, 0.5))
        col = tuple(float(x) for x in rng.uniform(0.3, 0.95, 3))
        name = 'm%02d' % k
        if mtype == DIFFUSE:
            mats.append(material(name, DIFFUSE, col, tex_albedo=0, tex_roughness=1, tex_bump=2))
        elif mtype == METAL:
            mats.append(material(name, METAL, col, sppm=False))
        elif mtype == GGX_CONDUCTOR:
            mats.append(material(name, GGX_CONDUCTOR, col, roughness=rough, index=1.1978, extinction=7.0488))
        else:
            mats.append(material(name, GGX_DIELECTRIC, (0.98, 0.98, 0.98), roughness=rough, index=1.5,
                                 opaque=False, sppm=False))
    base_p, base_n, base_uv = _displaced_sphere(rng, freq, 0.08)
    ext = float(extent)
    side = int(math.ceil(math.sqrt(instances)))
    cell = 2.0 * ext / side
    b = _Builder()
    b.quad((-ext, 0, -ext), (-ext, 0, ext), (ext, 0, ext), (ext, 0, -ext), (0, 1, 0), 0,
           uvs=((0, 0), (0, 8), (8, 8), (8, 0)))
    for k in range(instances):
        gx, gz = k % side, k // side
        rad = float(rng.uniform(0.2, 0.45)) * cell
        cx = -ext + (gx + 0.5) * cell + float(rng.uniform(-0.1, 0.1)) * cell
        cz = -ext + (gz + 0.5) * cell + float(rng.uniform(-0.1, 0.1)) * cell
        R = _rot_y(float(rng.uniform(0.0, 360.0)))
        pos = (base_p @ R.T) * rad + np.array([cx, 1.1 * rad + 1e-3, cz])
        b.tris(pos, base_n @ R.T, base_uv, 2 + k % 16)
    lh, ly = 0.3 * ext, 1.2 * ext
    b.quad((-lh, ly, -lh), (lh, ly, -lh), (lh, ly, lh), (-lh, ly, lh), (0, -1, 0), 1)
    scene = b.build()
    scene.update(materials=mats, textures=textures,
                 camera=_camera(THINLENS, width, height, (0.0, 0.55 * ext, -1.55 * ext), (0.0, 0.0, 0.1 * ext),
                                40.0, focal=0.9, dist=1.0, lens=aperture))
    return scene


def small_large_scene(seed=CONFIG_SEED_BASE + 104):
    """The large scene's construction at a size for tests: 16 copies of a
    2,000-triangle sphere, 64x36 pixels, 64^2 textures."""
    return large_scene(seed=seed, width=64, height=36, instances=16, freq=10, tex_size=64, light_tex=32)


BATCH_RESOLUTIONS = (128, 256, 512, 1024)


def batch_specs(seed=CONFIG_SEED_BASE + 3, count=64, tri_lo=10_000, tri_hi=2_000_000, photons_lo=50_000,
                photons_hi=1_000_000):
    """The batched workload's draw: per scene a triangle budget log-uniform
    over [tri_lo, tri_hi], a square resolution from BATCH_RESOLUTIONS and a
    photon count uniform over [photons_lo, photons_hi], plus a scene seed."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(count):
        tris = int(round(math.exp(rng.uniform(math.log(tri_lo), math.log(tri_hi)))))
        res = int(BATCH_RESOLUTIONS[int(rng.integers(0, len(BATCH_RESOLUTIONS)))])
        photons = int(rng.integers(photons_lo, photons_hi + 1))
        out.append(dict(triangles=tris, resolution=res, photons=photons, seed=int(rng.integers(0, 2 ** 62))))
    return out


def batch_scene(spec, tex_size=256, light_tex=64):
    """One scene of the batch: the mixed-materials construction (height field,
    spheres of the four surface types, textured field and light, thin lens)
    sized to the spec's triangle budget, half in the field and half in the
    spheres.  Textures are ``tex_size``^2 (the mixed-materials config's are
    1024^2) to keep the generation of 64 scenes short."""
    t = spec['triangles']
    field_n = max(8, int(math.sqrt(t / 4.0)) + 1)
    sphere_tris = max(0, t - 2 * (field_n - 1) ** 2)
    n_spheres = int(min(400, max(8, sphere_tris // 2376)))
    per = max(64, sphere_tris // n_spheres)
    n_lon = max(6, int(math.sqrt(per / 2.0)))
    n_lat = max(4, per // (2 * n_lon) + 1)
    res = spec['resolution']
    return mixed_materials(seed=spec['seed'], width=res, height=res, n_spheres=n_spheres, field_n=field_n,
                           tex_size=tex_size, light_tex=light_tex, n_lat=n_lat, n_lon=n_lon)


def demo_surface(k, name, rng):
    """Material k % 8 of the eight surface types, with the reference demo's
    parameters for the further four (main.cpp:14-114)."""
    t = k % 8
    col = tuple(float(x) for x in rng.uniform(0.3, 0.95, 3))
    rough = float(rng.uniform(0.05, 0.5))
    if t == DIFFUSE:
        return material(name, DIFFUSE, col)
    if t == METAL:
        return material(name, METAL, col, sppm=False)
    if t == GGX_CONDUCTOR:
        return material(name, GGX_CONDUCTOR, col, roughness=rough, index=1.1978, extinction=7.0488)
    if t == GGX_DIELECTRIC:
        return material(name, GGX_DIELECTRIC, (0.98, 0.98, 0.98), roughness=rough, index=1.5, opaque=False,
                        sppm=False)
    if t == BIMETAL:
        return material(name, BIMETAL, col, sppm=False)
    if t == GLASS:
        return material(name, GLASS, (0.98, 0.98, 0.98), index=1.5, opaque=False, sppm=False)
    if t == GLOSS_TRANSMIT:
        return material(name, GLOSS_TRANSMIT, (0.97, 0.98, 0.98), roughness=0.25, reflectance=0.1,
                        opaque=False, sppm=True)
    return material(name, DIFFUSE_TRANSMIT, col, reflectance=0.7, opaque=False, sppm=True)


def demo_materials(seed=CONFIG_SEED_BASE + 105, width=48, height=32, n_spheres=16, field_n=24, tex_size=64,
                   light_tex=32, n_lat=10, n_lon=12, aperture=0.05, extent=0.6):
    """The mixed-materials construction with spheres of all eight surface
    types in turn: the four of the mixed-materials config and the demo's
    BiMetal, Glass, GlossTransmit and DiffuseTransmit surfaces."""
    rng = np.random.Generator(np.random.PCG64(seed))
    textures = [noise_texture(rng, tex_size, 'albedo'), noise_texture(rng, tex_size, 'roughness'),
                noise_texture(rng, tex_size, 'normal'), noise_texture(rng, light_tex, 'emission')]
    mats = [material('field', DIFFUSE, (0.7, 0.7, 0.7), tex_albedo=0, tex_roughness=1, tex_bump=2),
            material('light', DIFFUSE, (1, 1, 1), emission=(10.0, 9.0, 8.0), tex_albedo=3)]
    b = _Builder()
    ext = float(extent)
    k_s = ext / 4.0
    height_field(b, rng, field_n, -ext, ext, -ext, ext, 0.25 * k_s, 0)
    for k in range(n_spheres):
        mats.append(demo_surface(k, 'd%03d' % k, rng))
        r = float(rng.uniform(0.05, 0.3)) * k_s
        cx, cz = rng.uniform(-ext * 0.85, ext * 0.85, 2)
        uv_sphere(b, (cx, 0.25 * k_s + r, cz), r, len(mats) - 1, n_lat, n_lon)
    ly, lh = 3.0 * k_s, 1.0 * k_s
    b.quad((-lh, ly, -lh), (lh, ly, -lh), (lh, ly, lh), (-lh, ly, lh), (0, -1, 0), 1)
    scene = b.build()
    scene.update(materials=mats, textures=textures,
                 camera=_camera(THINLENS, width, height, (0.0, 2.6 * k_s, -7.5 * k_s), (0.0, 0.2 * k_s, 0.0),
                                30.0, focal=0.9, dist=1.0, lens=aperture))
    return scene


def small_caustic(seed=CONFIG_SEED_BASE + 102, width=96, height=96):
    """The caustic scene at a size for tests: 12 coarser spheres, 96x96."""
    return caustic_box(seed=seed, width=width, height=height, n_spheres=12, n_lat=12, n_lon=16, light_tex=64)


def small_mixed(seed=CONFIG_SEED_BASE + 101, width=48, height=32, tex_size=64, ibl=False):
    """A small scene with every feature of the mixed-materials config (four
    material types, albedo/roughness/normal textures, textured light, thin
    lens) at a size the reference and the oracle finish in seconds.  ibl: an
    environment map (sky_texture) lights the paths that leave the scene."""
    scene = mixed_materials(seed=seed, width=width, height=height, n_spheres=12, field_n=24,
                            tex_size=tex_size, light_tex=32, n_lat=10, n_lon=12, aperture=0.05,
                            extent=0.6)
    if ibl:
        scene['ibl'] = sky_texture(np.random.Generator(np.random.PCG64(seed + 7)))
    return scene


def scene_stats(scene):
    return dict(triangles=int(len(scene['pos'])), materials=len(scene['materials']),
                textures=len(scene['textures']), width=scene['camera']['width'],
                height=scene['camera']['height'])
