"""Inputs for the watertight triangle test (FR_FLAG_WATERTIGHT): a closed
indexed mesh whose triangles share their vertices exactly, and rays from
inside it aimed exactly at its vertices and edge midpoints, where a
ray-triangle test that rounds differently on the two sides of an edge can let
a ray through."""
import numpy as np


def closed_mesh_scene(seed=7, n_lat=24, n_lon=32):
    """A bumpy UV sphere (one shared vertex array, so neighbouring triangles
    share their vertices bit for bit) around the origin, plus a small light
    triangle outside it; a pinhole camera inside."""
    import sys
    from frsppm import scenes
    rng = np.random.Generator(np.random.PCG64(seed))
    th = np.linspace(0.0, np.pi, n_lat + 1)
    ph = np.linspace(0.0, 2.0 * np.pi, n_lon, endpoint=False)
    verts = [np.array([0.0, 1.0, 0.0])]
    for i in range(1, n_lat):
        for j in range(n_lon):
            verts.append(np.array([np.sin(th[i]) * np.cos(ph[j]), np.cos(th[i]), np.sin(th[i]) * np.sin(ph[j])]))
    verts.append(np.array([0.0, -1.0, 0.0]))
    V = np.asarray(verts) * rng.uniform(0.8, 1.2, (len(verts), 1)) + np.array([0.1, -0.05, 0.07])
    V = V.astype(np.float32)

    def ring(i, j):
        return 1 + (i - 1) * n_lon + (j % n_lon)
    faces = []
    for j in range(n_lon):
        faces.append((0, ring(1, j + 1), ring(1, j)))
        faces.append((len(V) - 1, ring(n_lat - 1, j), ring(n_lat - 1, j + 1)))
    for i in range(1, n_lat - 1):
        for j in range(n_lon):
            a, b, c, d = ring(i, j), ring(i, j + 1), ring(i + 1, j), ring(i + 1, j + 1)
            faces.append((a, b, d))
            faces.append((a, d, c))
    F = np.asarray(faces, np.int64)
    pos = V[F]                                          # (T, 3, 3), shared vertices exact
    nrm = pos / np.linalg.norm(pos, axis=2, keepdims=True)
    light = np.array([[[3.0, 3.0, 3.0], [3.2, 3.0, 3.0], [3.0, 3.2, 3.0]]], np.float32)
    pos = np.concatenate([pos, light]).astype(np.float32)
    nrm = np.concatenate([nrm, np.tile([[[0.0, 0.0, 1.0]]], (1, 3, 1))]).astype(np.float32)
    uv = np.zeros((len(pos), 3, 2), np.float32)
    mat = np.zeros(len(pos), np.int32)
    mat[-1] = 1
    mats = [scenes.material('wall', scenes.DIFFUSE, (0.7, 0.7, 0.7)),
            scenes.material('light', scenes.DIFFUSE, (1.0, 1.0, 1.0), emission=(5.0, 5.0, 5.0))]
    cam = scenes._camera(scenes.PINHOLE, 16, 16, (0.1, -0.05, 0.07), (0.1, -0.05, 1.07), 60.0)
    return dict(pos=pos, nrm=nrm, uv=uv, mat=mat, materials=mats, textures=[], camera=cam), V, F


def edge_rays(V, F, center=(0.1, -0.05, 0.07)):
    """Rays (n x 7: origin, direction, index 1) from the centre toward every
    vertex and every edge midpoint of the mesh."""
    c = np.asarray(center, np.float32)
    targets = [V]
    for a, b in ((0, 1), (1, 2), (2, 0)):
        targets.append((V[F[:, a]] + V[F[:, b]]) * np.float32(0.5))
    T = np.concatenate(targets).astype(np.float32)
    d = T - c
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.broadcast_to(c, d.shape)
    return np.concatenate([o, d, np.ones((len(d), 1))], 1).astype(np.float32)
