"""ORACLE (test infrastructure only): ctypes binding of oracle/_build/libfrport.so,
the CPU restatement of the reference's SPPM path.  Used by tests/, smoke()
and bench.py's CPU baseline as the checker; never by the renderer."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, '_build', 'libfrport.so')

_f3 = C.c_float * 3


class PortMaterial(C.Structure):
    _fields_ = [('type', C.c_int32), ('sppm', C.c_int32), ('opaque', C.c_int32), ('tex_albedo', C.c_int32),
                ('tex_rough', C.c_int32), ('tex_bump', C.c_int32), ('albedo', _f3), ('emission', _f3),
                ('index', C.c_float), ('roughness', C.c_float), ('extinction', C.c_float),
                ('reflectance', C.c_float)]


class PortCamera(C.Structure):
    _fields_ = [('type', C.c_int32), ('width', C.c_int32), ('height', C.c_int32), ('pos', _f3), ('target', _f3),
                ('fov', C.c_float), ('focal', C.c_float), ('dist', C.c_float), ('aspect', C.c_float),
                ('lens', C.c_float)]


_libs = {}
_lib = None  # the float build (the parity restatement)

# Builds: 'f32' the parity restatement (the reference's float arithmetic),
# 'f64' the FP64 oracle (the same estimator in double, FR_PORT_REAL=double;
# its C API takes and returns doubles), 'timing' the restatement compiled
# with the reference's own optimisation flags for the CPU baseline.
LIBS = {'f32': LIB, 'f64': os.path.join(HERE, '_build', 'libfrport64.so'),
        'timing': os.path.join(HERE, '_build', 'libfrport_timing.so')}


def load(kind='f32'):
    global _lib
    if kind not in _libs:
        import importlib.util
        spec = importlib.util.spec_from_file_location('build_oracle', os.path.join(HERE, 'build_oracle.py'))
        m = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(m)
        m.build_port(kind)
        lib = C.CDLL(LIBS[kind])
        vp = C.c_void_p
        real = C.c_double if kind == 'f64' else C.c_float
        lib.port_create.restype = vp
        lib.port_create.argtypes = [C.c_int32, vp, vp, vp, vp, C.c_int32, vp, C.c_int32, vp, vp,
                                    C.POINTER(PortCamera), C.c_int32, real, real, C.c_int32]
        for name in ('port_destroy',):
            getattr(lib, name).argtypes = [vp]
            getattr(lib, name).restype = None
        lib.port_iterate.argtypes = [vp, C.c_int32]
        lib.port_set_ibl.argtypes = [vp, C.c_int32, C.c_int32, vp]
        lib.port_read_direct.argtypes = [vp, vp, vp, vp]
        lib.port_seek.argtypes = [vp, C.c_int32]
        lib.port_set_watertight.argtypes = [vp, C.c_int32]
        lib.port_set_stream_key.argtypes = [vp, C.c_uint32]
        lib.port_set_end_degenerate.argtypes = [vp, C.c_int32]
        lib.port_set_float_count.argtypes = [vp, C.c_int32]
        lib.port_set_window.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
        lib.port_sample_rays.argtypes = [vp, C.c_int64, C.c_int64]
        lib.port_read_ray_sample.argtypes = [vp, vp]
        lib.port_read_ray_sample.restype = C.c_int64
        lib.port_photon_pass.argtypes = [vp, C.c_int32, C.c_int32]
        lib.port_resolve.argtypes = [vp, vp]
        lib.port_trace_closest.argtypes = [vp, vp, C.c_int32, vp, vp]
        lib.port_trace_any.argtypes = [vp, vp, C.c_int32, vp]
        lib.port_read_hitpoints.argtypes = [vp] * 8
        lib.port_num_photons.argtypes = [vp]
        lib.port_num_photons.restype = C.c_int64
        lib.port_read_photons.argtypes = [vp, vp, vp, vp]
        lib.port_read_gather.argtypes = [vp, vp, vp]
        lib.port_read_state.argtypes = [vp, vp, vp, vp, vp]
        lib.port_radius_count.argtypes = [vp, C.c_int32, vp, C.c_int32, vp]
        lib.port_philox.argtypes = [vp, vp, vp]
        lib.port_set_threads.argtypes = [C.c_int32]
        lib.port_max_threads.restype = C.c_int32
        _libs[kind] = lib
        if kind == 'f32':
            _lib = lib
    return _libs[kind]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def set_threads(n):
    load().port_set_threads(int(n))


def max_threads():
    return int(load().port_max_threads())


def philox(ctr, key):
    out = np.zeros(4, np.uint32)
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    load().port_philox(_p(c), _p(k), _p(out))
    return out


def radius_count(hp_pos, hp_r, photons):
    hp = np.ascontiguousarray(np.concatenate([np.asarray(hp_pos, np.float32).reshape(-1, 3),
                                              np.asarray(hp_r, np.float32).reshape(-1, 1)], 1))
    ph = np.ascontiguousarray(photons, np.float32).reshape(-1, 3)
    out = np.empty(len(hp), np.int32)
    load().port_radius_count(_p(hp), len(hp), _p(ph), len(ph), _p(out))
    return out


class PortRenderer:
    """The CPU restatement on a scene dict from frsppm.scenes."""

    def __init__(self, scene, photons, alpha=0.9, radius=0.015, fix_stale=False, watertight=False, kind='f32',
                 float_count=False):
        """kind: 'f32' (the parity restatement), 'f64' (the FP64 oracle: its
        arrays are float64) or 'timing' (the reference's optimisation flags)."""
        lib = self.lib = load(kind)
        self.dt = dt = np.float64 if kind == 'f64' else np.float32
        self._keep = []
        pos = np.ascontiguousarray(scene['pos'], dt)
        nrm = np.ascontiguousarray(scene['nrm'], dt)
        uv = np.ascontiguousarray(scene['uv'], dt)
        mat = np.ascontiguousarray(scene['mat'], np.int32)
        texs = [np.ascontiguousarray(t, np.uint8) for t in scene['textures']]
        wh = np.array([[t.shape[1], t.shape[0]] for t in texs] or [[0, 0]], np.int32)
        tptr = (C.c_void_p * max(1, len(texs)))(*[t.ctypes.data for t in texs])
        mats = (PortMaterial * len(scene['materials']))()
        for k, m in enumerate(scene['materials']):
            d = mats[k]
            d.type, d.sppm, d.opaque = m['type'], int(m['sppm']), int(m['opaque'])
            d.tex_albedo, d.tex_rough, d.tex_bump = m['tex_albedo'], m['tex_roughness'], m['tex_bump']
            d.albedo = _f3(*m['albedo'])
            d.emission = _f3(*m['emission'])
            d.index, d.roughness, d.extinction, d.reflectance = m['index'], m['roughness'], m['extinction'], m['reflectance']
        c = scene['camera']
        cam = PortCamera(c['type'], c['width'], c['height'], _f3(*c['pos']), _f3(*c['target']), c['fov'],
                         c['focal'], c['dist'], c['aspect'], c['lens'])
        self._keep += [pos, nrm, uv, mat, texs, wh, tptr, mats]
        self.h = lib.port_create(len(pos), _p(pos), _p(nrm), _p(uv), _p(mat), len(scene['materials']), mats,
                                 len(texs), _p(wh), tptr, C.byref(cam), int(photons), float(alpha), float(radius),
                                 int(fix_stale))
        if not self.h:
            raise RuntimeError('port_create failed (no emissive facets?)')
        if watertight:
            lib.port_set_watertight(self.h, 1)
        if float_count:
            lib.port_set_float_count(self.h, 1)
        if scene.get('ibl') is not None:
            ibl = np.ascontiguousarray(scene['ibl'], np.uint8)
            lib.port_set_ibl(self.h, ibl.shape[1], ibl.shape[0], _p(ibl))
        self.width, self.height, self.photons = c['width'], c['height'], int(photons)

    def close(self):
        if getattr(self, 'h', None):
            self.lib.port_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def iterate(self, n=1):
        self.lib.port_iterate(self.h, int(n))

    def seek(self, first_step):
        """The next iteration runs step first_step + 1."""
        self.lib.port_seek(self.h, int(first_step))

    def sample_rays(self, stride, cap):
        """Keep every stride-th closest-hit ray the next iterations trace (up to cap)."""
        self.lib.port_sample_rays(self.h, int(stride), int(cap))

    def ray_sample(self):
        """The kept rays: (N x 7 float32 {origin, direction, index}, N pass tags 0 eye / 1 photon)."""
        n = int(self.lib.port_read_ray_sample(self.h, None))
        out = np.empty((n, 8), self.dt)
        self.lib.port_read_ray_sample(self.h, _p(out))
        return np.ascontiguousarray(out[:, :7]), out[:, 7].astype(np.int32)

    def photon_pass(self, first, count):
        self.lib.port_photon_pass(self.h, int(first), int(count))

    def resolve(self):
        out = np.empty((self.width * self.height, 4), self.dt)
        self.lib.port_resolve(self.h, _p(out))
        return out

    def trace_closest(self, rays):
        rays = np.ascontiguousarray(rays, self.dt).reshape(-1, 7)
        f = np.empty(len(rays), np.int32)
        tuv = np.empty((len(rays), 3), self.dt)
        self.lib.port_trace_closest(self.h, _p(rays), len(rays), _p(f), _p(tuv))
        return f, tuv

    def trace_any(self, rays):
        rays = np.ascontiguousarray(rays, self.dt).reshape(-1, 8)
        hit = np.empty(len(rays), np.int32)
        self.lib.port_trace_any(self.h, _p(rays), len(rays), _p(hit))
        return hit

    def read_hitpoints(self):
        n = self.width * self.height
        t, f = np.empty(n, np.int32), np.empty(n, np.int32)
        a = [np.empty((n, 3), self.dt) for _ in range(4)]
        rough = np.empty(n, self.dt)
        self.lib.port_read_hitpoints(self.h, _p(t), _p(f), *[_p(x) for x in a], _p(rough))
        return dict(type=t, facet=f, pos=a[0], nrm=a[1], out=a[2], w=a[3], rough=rough)

    def read_direct(self):
        """Direct (environment) light: per hitpoint of the last iteration, and
        per pixel the sum and count (SharedHitPoint::DirectLight, NumDirectLight)."""
        n = self.width * self.height
        hp, sp = np.empty((n, 3), self.dt), np.empty((n, 3), self.dt)
        cnt = np.empty(n, np.int32)
        self.lib.port_read_direct(self.h, _p(hp), _p(sp), _p(cnt))
        return hp, sp, cnt

    def compacted_photons(self):
        n = int(self.lib.port_num_photons(self.h))
        ph = np.empty((n, 11), self.dt)
        path, slot = np.empty(n, np.int32), np.empty(n, np.int32)
        self.lib.port_read_photons(self.h, _p(ph), _p(path), _p(slot))
        return ph, path, slot

    def read_gather(self):
        n = self.width * self.height
        m = np.empty(n, np.int32)
        phi = np.empty((n, 3), self.dt)
        self.lib.port_read_gather(self.h, _p(m), _p(phi))
        return m, phi

    def read_state(self):
        n = self.width * self.height
        rad = np.empty((n, 3), self.dt)
        N, r, g = np.empty(n, np.int32), np.empty(n, self.dt), np.empty(n, np.int32)
        self.lib.port_read_state(self.h, _p(rad), _p(N), _p(r), _p(g))
        return dict(tau=rad, n=N, r=r, g=g)
