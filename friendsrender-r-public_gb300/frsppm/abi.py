"""ctypes binding of the C-ABI in include/friendsrender.h (libfrsppm.so).

``Renderer`` wraps one fr_ctx.  Loading fails loudly when the library is
missing: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

FR_OK = 0

_f3 = C.c_float * 3


class MaterialDesc(C.Structure):
    _fields_ = [('type', C.c_int32), ('sppm_surface', C.c_int32), ('opaque', C.c_int32),
                ('tex_albedo', C.c_int32), ('tex_roughness', C.c_int32), ('tex_bump', C.c_int32),
                ('albedo', _f3), ('emission', _f3), ('index', C.c_float), ('roughness', C.c_float),
                ('extinction', C.c_float), ('reflectance', C.c_float)]


class TextureDesc(C.Structure):
    _fields_ = [('width', C.c_int32), ('height', C.c_int32), ('texels', C.c_void_p)]


class SceneDesc(C.Structure):
    _fields_ = [('num_facets', C.c_int32), ('positions', C.c_void_p), ('normals', C.c_void_p),
                ('uvs', C.c_void_p), ('material_ids', C.c_void_p), ('num_materials', C.c_int32),
                ('materials', C.POINTER(MaterialDesc)), ('num_textures', C.c_int32),
                ('textures', C.POINTER(TextureDesc)), ('environment', C.POINTER(TextureDesc))]


class CameraDesc(C.Structure):
    _fields_ = [('type', C.c_int32), ('width', C.c_int32), ('height', C.c_int32), ('position', _f3),
                ('target', _f3), ('fov_degrees', C.c_float), ('focal_length', C.c_float),
                ('distance_to_lens', C.c_float), ('aspect', C.c_float), ('lens_width', C.c_float),
                ('lens_height', C.c_float)]


class SPPMParams(C.Structure):
    _fields_ = [('photons_per_iteration', C.c_int32), ('alpha', C.c_float), ('initial_radius', C.c_float),
                ('flags', C.c_uint32), ('grid_cell_scale', C.c_float), ('guide', C.c_int32),
                ('guide_plain_fraction', C.c_float), ('guide_batch', C.c_int32),
                ('guide_learning_rate', C.c_float), ('guide_seed', C.c_uint32),
                ('guide_steps', C.c_int32), ('bvh_builder', C.c_int32)]


# fr_material_fn: int (*)(void* user, const char* name, fr_material_desc* material)
MATERIAL_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_char_p, C.POINTER(MaterialDesc))
FR_ERR_IO = 5

GUIDE_PARAMS = 11824
FLAG_FIX_STALE_PHOTON_SLOT = 1   # FR_FLAG_FIX_STALE_PHOTON_SLOT
FLAG_STANDARD_RESOLVE = 2        # FR_FLAG_STANDARD_RESOLVE
FLAG_END_DEGENERATE_PATHS = 4    # FR_FLAG_END_DEGENERATE_PATHS
FLAG_WATERTIGHT = 8              # FR_FLAG_WATERTIGHT
FLAG_FLOAT_PHOTON_COUNT = 16     # FR_FLAG_FLOAT_PHOTON_COUNT
BVH_HOST_SAH, BVH_DEVICE_LBVH = 0, 1  # FR_BVH_*


class Stats(C.Structure):
    _fields_ = [('iterations', C.c_int64), ('photon_paths', C.c_int64), ('pixels', C.c_int64),
                ('triangles', C.c_int64), ('bvh_nodes', C.c_int64), ('photon_table', C.c_int64),
                ('device_bytes', C.c_double)]


# Every symbol include/friendsrender.h declares.
EXPORTS = ['fr_last_error', 'fr_create', 'fr_iterate', 'fr_synchronize', 'fr_resolve', 'fr_resolve_dev',
           'fr_get_stats', 'fr_stream', 'fr_destroy', 'fr_trace_closest', 'fr_trace_any', 'fr_radius_query',
           'fr_read_hitpoints', 'fr_read_photon_slots', 'fr_read_gather', 'fr_read_state', 'fr_profile_enable',
           'fr_profile_read', 'fr_radius_count_noalloc', 'fr_check_exact_math',
           'fr_read_wave_counts', 'fr_save_state', 'fr_load_state', 'fr_update',
           'fr_resolve_rgba8', 'fr_export_png', 'fr_write_png', 'fr_check_tc_gemm', 'fr_guide_params',
           'fr_guide_set_params', 'fr_read_guide_importance', 'fr_guide_gradient', 'fr_seek', 'fr_iterate_batch',
           'fr_autotune', 'fr_update_dev', 'fr_read_direct', 'fr_scene_load_obj', 'fr_scene_get_desc',
           'fr_scene_material_name', 'fr_scene_free', 'fr_texture_load', 'fr_resolve_async', 'fr_resolve_wait',
           'fr_batch_create', 'fr_batch_iterate', 'fr_batch_destroy']

STAGES = ('eye', 'photon', 'grid', 'gather', 'eye_trace', 'photon_trace')

_lib = None


def load(path=None):
    """Load libfrsppm.so (built in-tree by frsppm.build)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or _build.LIB
    if not os.path.exists(path):
        raise RuntimeError('libfrsppm.so not built (%s); run __graft_entry__.build()' % path)
    lib = C.CDLL(path)
    vp, i32, f32 = C.c_void_p, C.c_int32, C.c_float
    lib.fr_last_error.restype = C.c_char_p
    lib.fr_create.argtypes = [C.POINTER(SceneDesc), C.POINTER(CameraDesc), C.POINTER(SPPMParams), C.POINTER(vp)]
    lib.fr_iterate.argtypes = [vp, C.c_int]
    lib.fr_synchronize.argtypes = [vp]
    lib.fr_resolve.argtypes = [vp, vp]
    lib.fr_resolve_dev.argtypes = [vp, vp]
    lib.fr_resolve_async.argtypes = [vp, vp, C.POINTER(C.c_uint64)]
    lib.fr_resolve_wait.argtypes = [vp, C.c_uint64]
    lib.fr_get_stats.argtypes = [vp, C.POINTER(Stats)]
    lib.fr_stream.argtypes = [vp]
    lib.fr_stream.restype = vp
    lib.fr_destroy.argtypes = [vp]
    lib.fr_destroy.restype = None
    lib.fr_trace_closest.argtypes = [vp, vp, i32, vp, vp]
    lib.fr_trace_any.argtypes = [vp, vp, i32, vp]
    lib.fr_radius_query.argtypes = [vp, vp, i32, vp, i32, f32, vp, vp, C.c_uint32, vp]
    lib.fr_read_hitpoints.argtypes = [vp, vp, vp, vp, vp]
    lib.fr_read_photon_slots.argtypes = [vp, vp, vp, vp, vp]
    lib.fr_read_gather.argtypes = [vp, vp, vp]
    lib.fr_read_state.argtypes = [vp, vp, vp, vp, vp]
    lib.fr_profile_enable.argtypes = [vp, i32, i32]
    lib.fr_profile_read.argtypes = [vp, vp, vp, vp]
    lib.fr_radius_count_noalloc.argtypes = [vp, i32, vp, i32, f32, vp, vp]
    lib.fr_check_exact_math.argtypes = [C.c_uint64, C.c_uint32, vp, vp]
    lib.fr_read_wave_counts.argtypes = [vp, vp, vp, vp, vp]
    lib.fr_save_state.argtypes = [vp, vp, C.POINTER(C.c_size_t)]
    lib.fr_load_state.argtypes = [vp, vp, C.c_size_t]
    lib.fr_seek.argtypes = [vp, C.c_uint32]
    lib.fr_iterate_batch.argtypes = [C.POINTER(vp), C.c_int, C.c_int]
    lib.fr_autotune.argtypes = [vp, C.c_int, C.POINTER(C.c_uint32)]
    lib.fr_update.argtypes = [vp, vp, vp]
    lib.fr_update_dev.argtypes = [vp, vp, vp]
    lib.fr_read_direct.argtypes = [vp, vp, vp, vp]
    lib.fr_resolve_rgba8.argtypes = [vp, vp]
    lib.fr_export_png.argtypes = [vp, C.c_char_p]
    lib.fr_write_png.argtypes = [C.c_char_p, i32, i32, vp]
    lib.fr_check_tc_gemm.argtypes = [C.c_uint32, vp]
    lib.fr_guide_params.argtypes = [vp, vp]
    lib.fr_guide_set_params.argtypes = [vp, vp]
    lib.fr_read_guide_importance.argtypes = [vp, vp]
    lib.fr_guide_gradient.argtypes = [vp, i32, vp, vp, vp]
    lib.fr_scene_load_obj.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, MATERIAL_FN, vp, C.POINTER(vp)]
    lib.fr_scene_get_desc.argtypes = [vp]
    lib.fr_scene_get_desc.restype = C.POINTER(SceneDesc)
    lib.fr_scene_material_name.argtypes = [vp, i32]
    lib.fr_scene_material_name.restype = C.c_char_p
    lib.fr_scene_free.argtypes = [vp]
    lib.fr_scene_free.restype = None
    lib.fr_texture_load.argtypes = [C.c_char_p, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), vp]
    lib.fr_batch_create.argtypes = [C.POINTER(vp), C.c_int, C.POINTER(vp)]
    lib.fr_batch_iterate.argtypes = [vp, C.c_int]
    lib.fr_batch_destroy.argtypes = [vp]
    lib.fr_batch_destroy.restype = None
    _lib = lib
    return lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _check(rc, what):
    if rc != FR_OK:
        msg = _lib.fr_last_error().decode() if _lib else ''
        raise RuntimeError('%s failed (%d): %s' % (what, rc, msg))


class Renderer:
    """One fr_ctx: a scene (frsppm.scenes dict), camera and SPPM parameters."""

    def __init__(self, scene, photons, alpha=0.9, radius=0.015, flags=0, cell_scale=0.0, camera=None,
                 guide=False, guide_plain_fraction=0.0, guide_batch=0, guide_lr=0.0, guide_seed=1, guide_steps=0,
                 bvh_builder=0):
        lib = load()
        self.scene = scene
        cam = camera or scene['camera']
        self._keep = []
        pos = np.ascontiguousarray(scene['pos'], np.float32)
        nrm = np.ascontiguousarray(scene['nrm'], np.float32)
        uv = np.ascontiguousarray(scene['uv'], np.float32)
        mat = np.ascontiguousarray(scene['mat'], np.int32)
        texs = [np.ascontiguousarray(t, np.uint8) for t in scene['textures']]
        self._keep += [pos, nrm, uv, mat] + texs
        mats = (MaterialDesc * len(scene['materials']))()
        for k, m in enumerate(scene['materials']):
            d = mats[k]
            d.type, d.sppm_surface, d.opaque = m['type'], int(m['sppm']), int(m['opaque'])
            d.tex_albedo, d.tex_roughness, d.tex_bump = m['tex_albedo'], m['tex_roughness'], m['tex_bump']
            d.albedo = _f3(*m['albedo'])
            d.emission = _f3(*m['emission'])
            d.index, d.roughness, d.extinction, d.reflectance = m['index'], m['roughness'], m['extinction'], m['reflectance']
        tds = (TextureDesc * max(1, len(texs)))()
        for k, t in enumerate(texs):
            tds[k].width, tds[k].height = t.shape[1], t.shape[0]
            tds[k].texels = t.ctypes.data
        self._keep += [mats, tds]
        sd = SceneDesc(len(pos), pos.ctypes.data, nrm.ctypes.data, uv.ctypes.data, mat.ctypes.data,
                       len(scene['materials']), mats, len(texs), tds)
        if scene.get('ibl') is not None:  # environment map
            env = np.ascontiguousarray(scene['ibl'], np.uint8)
            ed = TextureDesc(env.shape[1], env.shape[0], env.ctypes.data)
            self._keep += [env, ed]
            sd.environment = C.pointer(ed)
        cd = CameraDesc()
        cd.type, cd.width, cd.height = cam['type'], cam['width'], cam['height']
        cd.position = _f3(*cam['pos'])
        cd.target = _f3(*cam['target'])
        cd.fov_degrees, cd.focal_length, cd.distance_to_lens = cam['fov'], cam['focal'], cam['dist']
        cd.aspect = cam['aspect']
        cd.lens_width = cd.lens_height = cam['lens']
        pp = SPPMParams(int(photons), float(alpha), float(radius), int(flags), float(cell_scale), int(bool(guide)),
                        float(guide_plain_fraction), int(guide_batch), float(guide_lr), int(guide_seed),
                        int(guide_steps), int(bvh_builder))
        self.width, self.height, self.photons = cam['width'], cam['height'], int(photons)
        h = C.c_void_p()
        _check(lib.fr_create(C.byref(sd), C.byref(cd), C.byref(pp), C.byref(h)), 'fr_create')
        self.h = h

    def close(self):
        if getattr(self, 'h', None):
            _lib.fr_destroy(self.h)
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

    def iterate(self, n=1, sync=True):
        _check(_lib.fr_iterate(self.h, int(n)), 'fr_iterate')
        if sync:
            self.synchronize()

    def synchronize(self):
        _check(_lib.fr_synchronize(self.h), 'fr_synchronize')

    def stream(self):
        return _lib.fr_stream(self.h)

    def profile(self, on, max_iterations=256):
        _check(_lib.fr_profile_enable(self.h, int(on), int(max_iterations)), 'fr_profile_enable')

    def profile_read(self):
        ms = np.zeros(len(STAGES), np.float64)
        cnt = np.zeros(len(STAGES), np.int64)
        launches = np.zeros(1, np.int64)
        _check(_lib.fr_profile_read(self.h, _ptr(ms), _ptr(cnt), _ptr(launches)), 'fr_profile_read')
        return dict(zip(STAGES, ms.tolist())), dict(zip(STAGES, cnt.tolist())), int(launches[0])

    def resolve(self):
        out = np.empty((self.width * self.height, 4), np.float32)
        _check(_lib.fr_resolve(self.h, _ptr(out)), 'fr_resolve')
        return out

    def resolve_dev(self, dev_ptr):
        _check(_lib.fr_resolve_dev(self.h, C.c_void_p(dev_ptr)), 'fr_resolve_dev')

    def resolve_async(self, host_ptr):
        """fr_resolve_async into the host buffer at host_ptr (width*height*4
        floats, best pinned); returns the ticket for resolve_wait."""
        t = C.c_uint64()
        _check(_lib.fr_resolve_async(self.h, C.c_void_p(host_ptr), C.byref(t)), 'fr_resolve_async')
        return t.value

    def resolve_wait(self, ticket):
        _check(_lib.fr_resolve_wait(self.h, C.c_uint64(ticket)), 'fr_resolve_wait')

    def stats(self):
        s = Stats()
        _check(_lib.fr_get_stats(self.h, C.byref(s)), 'fr_get_stats')
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def trace_closest(self, rays):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 7)
        n = len(rays)
        facet = np.empty(n, np.int32)
        tuv = np.empty((n, 3), np.float32)
        _check(_lib.fr_trace_closest(self.h, _ptr(rays), n, _ptr(facet), _ptr(tuv)), 'fr_trace_closest')
        return facet, tuv

    def trace_any(self, rays):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        hit = np.empty(len(rays), np.int32)
        _check(_lib.fr_trace_any(self.h, _ptr(rays), len(rays), _ptr(hit)), 'fr_trace_any')
        return hit

    def radius_query(self, hp_pos, hp_r, photons, cell, pairs_capacity=0):
        hp = np.ascontiguousarray(np.concatenate([np.asarray(hp_pos, np.float32).reshape(-1, 3),
                                                  np.asarray(hp_r, np.float32).reshape(-1, 1)], 1))
        ph = np.ascontiguousarray(photons, np.float32).reshape(-1, 3)
        counts = np.empty(len(hp), np.int32)
        pairs = np.empty((max(pairs_capacity, 1), 2), np.uint32) if pairs_capacity else None
        pc = np.zeros(1, np.uint32)
        _check(_lib.fr_radius_query(self.h, _ptr(hp), len(hp), _ptr(ph), len(ph), float(cell), _ptr(counts),
                                    _ptr(pairs), int(pairs_capacity), _ptr(pc) if pairs is not None else None),
               'fr_radius_query')
        if pairs is None:
            return counts, None
        return counts, pairs[:min(int(pc[0]), pairs_capacity)]

    def read_hitpoints(self):
        n = self.width * self.height
        a = [np.empty((n, 4), np.float32) for _ in range(4)]
        _check(_lib.fr_read_hitpoints(self.h, *[_ptr(x) for x in a]), 'fr_read_hitpoints')
        pos, nrm, out, wgt = a
        return dict(type=pos[:, 3].view(np.int32).copy(), pos=pos[:, :3].copy(), nrm=nrm[:, :3].copy(),
                    rough=nrm[:, 3].copy(), out=out[:, :3].copy(), mat=out[:, 3].view(np.int32).copy(),
                    w=wgt[:, :3].copy(), facet=wgt[:, 3].view(np.int32).copy())

    def read_photon_slots(self):
        n = self.photons * 32
        a = [np.empty((n, 4), np.float32) for _ in range(3)]
        counts = np.empty(self.photons, np.uint32)
        _check(_lib.fr_read_photon_slots(self.h, *[_ptr(x) for x in a], _ptr(counts)), 'fr_read_photon_slots')
        return a[0], a[1], a[2], counts

    def compacted_photons(self):
        """Photons of the last iteration in the compactor's order (path, slot):
        (N, 11) {pos, flux, indir, index, pdf}, path ids and slot ids."""
        pos, flux, d, counts = self.read_photon_slots()
        paths = np.repeat(np.arange(self.photons), counts.astype(np.int64))
        slots = np.concatenate([np.arange(c) for c in counts]) if len(counts) else np.zeros(0, int)
        idx = paths * 32 + slots
        ph = np.concatenate([pos[idx, :3], flux[idx, :3], d[idx, :3], pos[idx, 3:4], flux[idx, 3:4]], 1)
        return ph, paths.astype(np.int32), slots.astype(np.int32)

    def wave_counts(self):
        """Paths traced per round of the last iteration's eye and photon
        passes, and (last entry) the paths handed to each tail kernel."""
        e = np.zeros(17, np.uint32)
        p = np.zeros(17, np.uint32)
        er = np.zeros(1, np.int32)
        pr = np.zeros(1, np.int32)
        _check(_lib.fr_read_wave_counts(self.h, _ptr(e), _ptr(p), _ptr(er), _ptr(pr)), 'fr_read_wave_counts')
        return e[:er[0] + 1].copy(), p[:pr[0] + 1].copy()

    def save_state(self):
        """Checkpoint of the iteration state (bytes)."""
        n = C.c_size_t(0)
        _check(_lib.fr_save_state(self.h, None, C.byref(n)), 'fr_save_state')
        buf = np.empty(n.value, np.uint8)
        _check(_lib.fr_save_state(self.h, _ptr(buf), C.byref(n)), 'fr_save_state')
        return buf[:n.value].tobytes()

    def load_state(self, data):
        buf = np.frombuffer(data, np.uint8)
        _check(_lib.fr_load_state(self.h, _ptr(buf), len(buf)), 'fr_load_state')

    def autotune(self, iterations=2):
        """fr_autotune: runs 5 * (iterations + 1) iterations; returns the chosen threshold."""
        out = C.c_uint32(0)
        _check(_lib.fr_autotune(self.h, int(iterations), C.byref(out)), 'fr_autotune')
        return int(out.value)

    def seek(self, first_step):
        """fr_seek: iteration k of this (fresh) context draws step first_step + k."""
        _check(_lib.fr_seek(self.h, int(first_step)), 'fr_seek')

    def read_direct(self):
        """fr_read_direct: (last iteration's per-pixel direct light, per-pixel sums, counts)."""
        n = self.width * self.height
        last, tot = np.empty((n, 3), np.float32), np.empty((n, 3), np.float32)
        cnt = np.empty(n, np.int32)
        _check(_lib.fr_read_direct(self.h, _ptr(last), _ptr(tot), _ptr(cnt)), 'fr_read_direct')
        return last, tot, cnt

    def update_dev(self, m_ptr, phi4_ptr, sync=True):
        """fr_update_dev: device pointers to width*height int32 M and float4 flux sums."""
        _check(_lib.fr_update_dev(self.h, C.c_void_p(m_ptr), C.c_void_p(phi4_ptr)), 'fr_update_dev')
        if sync:
            self.synchronize()

    def update(self, m, phi):
        """fr_update: apply per-pixel photon counts and flux sums to the state."""
        m = np.ascontiguousarray(m, np.int32)
        phi = np.ascontiguousarray(phi, np.float32)
        _check(_lib.fr_update(self.h, _ptr(m), _ptr(phi)), 'fr_update')

    def resolve_rgba8(self):
        """ExportPNG's pixels: (height, width, 4) uint8."""
        out = np.empty((self.height, self.width, 4), np.uint8)
        _check(_lib.fr_resolve_rgba8(self.h, _ptr(out)), 'fr_resolve_rgba8')
        return out

    def export_png(self, path):
        _check(_lib.fr_export_png(self.h, os.fsencode(path)), 'fr_export_png')

    def guide_params(self):
        out = np.empty(GUIDE_PARAMS, np.float32)
        _check(_lib.fr_guide_params(self.h, _ptr(out)), 'fr_guide_params')
        return out

    def set_guide_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        assert p.shape == (GUIDE_PARAMS,)
        _check(_lib.fr_guide_set_params(self.h, _ptr(p)), 'fr_guide_set_params')

    def guide_importance(self):
        out = np.empty(self.photons, np.float32)
        _check(_lib.fr_read_guide_importance(self.h, _ptr(out)), 'fr_read_guide_importance')
        return out

    def guide_gradient(self, samples):
        """samples: (n, 9) float32 {5 inputs, direction, importance}; returns
        (gradient sums (GUIDE_PARAMS,), importance sum)."""
        smp = np.ascontiguousarray(samples, np.float32).reshape(-1, 9)
        grad = np.empty(GUIDE_PARAMS, np.float32)
        ws = np.zeros(1, np.float32)
        _check(_lib.fr_guide_gradient(self.h, len(smp), _ptr(smp), _ptr(grad), _ptr(ws)), 'fr_guide_gradient')
        return grad, float(ws[0])

    def read_gather(self):
        n = self.width * self.height
        m = np.empty(n, np.int32)
        phi = np.empty((n, 4), np.float32)
        _check(_lib.fr_read_gather(self.h, _ptr(m), _ptr(phi)), 'fr_read_gather')
        return m, phi[:, :3].copy()

    def read_state(self):
        n = self.width * self.height
        tau = np.empty((n, 3), np.float64)
        N = np.empty(n, np.int32)
        r = np.empty(n, np.float32)
        g = np.empty(n, np.int32)
        _check(_lib.fr_read_state(self.h, _ptr(tau), _ptr(N), _ptr(r), _ptr(g)), 'fr_read_state')
        return dict(tau=tau, n=N, r=r, g=g)


EXACT_FUNCTIONS = ('pow_m2', 'ggx_cth', 'ggx_pdf', 'glass_cth', 'glass_pdf', 'metal_brdf', 'conductor_lambda',
                   'conductor_tm3', 'sqrt_half')


def check_exact_math(samples, seed=1):
    """fr_check_exact_math: {function: (fast-path count, mismatches)}."""
    lib = load()
    mm = np.zeros(len(EXACT_FUNCTIONS), np.uint64)
    fp = np.zeros(len(EXACT_FUNCTIONS), np.uint64)
    _check(lib.fr_check_exact_math(int(samples), int(seed), _ptr(mm), _ptr(fp)), 'fr_check_exact_math')
    return {n: (int(fp[k]), int(mm[k])) for k, n in enumerate(EXACT_FUNCTIONS)}


def write_png(path, rgba):
    """fr_write_png: (height, width, 4) uint8 to a PNG file (no GPU needed)."""
    lib = load()
    rgba = np.ascontiguousarray(rgba, np.uint8)
    h, w = rgba.shape[:2]
    rc = lib.fr_write_png(os.fsencode(path), w, h, _ptr(rgba))
    if rc != FR_OK:
        raise RuntimeError('fr_write_png failed (%d)' % rc)


def check_tc_gemm(seed=1):
    """fr_check_tc_gemm: max |error| of the three tcgen05 products."""
    lib = load()
    err = np.zeros(3, np.float64)
    _check(lib.fr_check_tc_gemm(int(seed), _ptr(err)), 'fr_check_tc_gemm')
    return err


class Batch:
    """fr_batch_create over Renderer objects: one CUDA graph holding one
    iteration of every scene; iterate(n) launches it n times."""

    def __init__(self, renderers):
        self.renderers = list(renderers)
        arr = (C.c_void_p * len(self.renderers))(*[r.h.value if isinstance(r.h, C.c_void_p) else r.h
                                                   for r in self.renderers])
        self.h = C.c_void_p()
        _check(_lib.fr_batch_create(arr, len(self.renderers), C.byref(self.h)), 'fr_batch_create')

    def iterate(self, n=1, sync=True):
        _check(_lib.fr_batch_iterate(self.h, int(n)), 'fr_batch_iterate')
        if sync:
            for r in self.renderers:
                r.synchronize()

    def close(self):
        if getattr(self, 'h', None):
            _lib.fr_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def iterate_batch(renderers, n=1, sync=True):
    """fr_iterate_batch over Renderer objects (n iterations of each)."""
    arr = (C.c_void_p * len(renderers))(*[r.h.value if isinstance(r.h, C.c_void_p) else r.h for r in renderers])
    _check(_lib.fr_iterate_batch(arr, len(renderers), int(n)), 'fr_iterate_batch')
    if sync:
        for r in renderers:
            r.synchronize()



# ------------------------------------------------------------------ scene ingest

_MATERIAL_FIELDS = ('type', 'sppm', 'opaque', 'index', 'roughness', 'extinction', 'reflectance')


def load_texture(path):
    """fr_texture_load: (H x W x 4 uint8 RGBA8, channel count stbi_load reports)."""
    lib = load()
    w, h, c = C.c_int32(), C.c_int32(), C.c_int32()
    _check(lib.fr_texture_load(os.fsencode(path), C.byref(w), C.byref(h), C.byref(c), None), 'fr_texture_load')
    out = np.empty((h.value, w.value, 4), np.uint8)
    _check(lib.fr_texture_load(os.fsencode(path), None, None, None, _ptr(out)), 'fr_texture_load')
    return out, c.value


def load_obj_scene(obj_file, asset_dir=None, environment=None, materials=None):
    """fr_scene_load_obj: Scene::CreateScene on an OBJ file, as a scene dict
    (the layout frsppm.scenes makes, without a camera).

    ``materials`` is the material plug-in (SceneMaterialManager): None keeps
    the loader's defaults, a dict maps material names to dicts of any of
    type, sppm, opaque, index, roughness, extinction, reflectance (names not
    in it keep the defaults), and a callable f(name, fields) may change the
    ``fields`` dict (the same keys plus albedo and emission) in place."""
    lib = load()
    errors = []

    def plugin(_user, name, desc):
        try:
            d = desc.contents
            name = name.decode()
            fields = dict(type=d.type, sppm=d.sppm_surface, opaque=d.opaque, index=d.index,
                          roughness=d.roughness, extinction=d.extinction, reflectance=d.reflectance,
                          albedo=tuple(d.albedo), emission=tuple(d.emission))
            if callable(materials):
                materials(name, fields)
            elif name in materials:
                fields.update(materials[name])
            d.type, d.sppm_surface, d.opaque = int(fields['type']), int(fields['sppm']), int(fields['opaque'])
            d.index, d.roughness = float(fields['index']), float(fields['roughness'])
            d.extinction, d.reflectance = float(fields['extinction']), float(fields['reflectance'])
            d.albedo = _f3(*fields['albedo'])
            d.emission = _f3(*fields['emission'])
            return 0
        except Exception as e:  # reported after the call; the loader sees a failure
            errors.append(e)
            return 1

    cb = MATERIAL_FN(plugin) if materials is not None else MATERIAL_FN()
    h = C.c_void_p()
    rc = lib.fr_scene_load_obj(os.fsencode(obj_file), None if asset_dir is None else os.fsencode(asset_dir),
                               None if environment is None else os.fsencode(environment), cb, None, C.byref(h))
    if errors:
        raise errors[0]
    _check(rc, 'fr_scene_load_obj')
    try:
        d = lib.fr_scene_get_desc(h).contents
        t = d.num_facets

        def arr(ptr, ctype, shape):
            n = int(np.prod(shape))
            if n == 0:
                return np.zeros(shape, np.dtype(ctype))
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), (n,)).reshape(shape).copy()

        scene = dict(pos=arr(d.positions, C.c_float, (t, 3, 3)), nrm=arr(d.normals, C.c_float, (t, 3, 3)),
                     uv=arr(d.uvs, C.c_float, (t, 3, 2)), mat=arr(d.material_ids, C.c_int32, (t,)))
        mats = []
        for m in range(d.num_materials):
            md = d.materials[m]
            mats.append(dict(name=lib.fr_scene_material_name(h, m).decode(), type=md.type, sppm=bool(md.sppm_surface),
                             opaque=bool(md.opaque), tex_albedo=md.tex_albedo, tex_roughness=md.tex_roughness,
                             tex_bump=md.tex_bump, albedo=tuple(md.albedo), emission=tuple(md.emission),
                             index=md.index, roughness=md.roughness, extinction=md.extinction,
                             reflectance=md.reflectance))
        scene['materials'] = mats
        scene['textures'] = [arr(d.textures[k].texels, C.c_uint8, (d.textures[k].height, d.textures[k].width, 4))
                             for k in range(d.num_textures)]
        if d.environment:
            e = d.environment.contents
            scene['ibl'] = arr(e.texels, C.c_uint8, (e.height, e.width, 4))
        else:
            scene['ibl'] = None
        return scene
    finally:
        lib.fr_scene_free(h)
