"""Benchmark: SPPM iterations of the mixed-materials workload on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one SPPM iteration (eye pass over every pixel, photon pass of the
iteration's photon paths, photon grid build, gather + N/tau/R update) of the
mixed-materials scene: 997,444 triangles (200 seeded UV spheres + a 512^2
value-noise height field), diffuse / specular / GGX conductor / GGX
dielectric materials, 1024^2 albedo/roughness/normal textures, a 512^2
textured area light, a 1280x720 thin-lens camera (aperture 0.02), 1M photon
paths per iteration, alpha 0.7, initial radius 0.02.

value: photon paths/s over all GPUs, inputs resident in HBM, CUDA events on
the renderer's stream, L2 flushed (256 MB write) before every timed step.
Stage times and the roofline come from a second, profiled run of the same
steps (CUDA events around every stage and trace launch).
e2e: the same metric through the C-ABI with host result buffers: every step
is fr_iterate + fr_resolve_async into pinned host memory (the image, read back
each step, two buffers in turn) and a wait for the previous step's image, so
the copy overlaps the next iteration; the scene is uploaded once by fr_create
(reported as setup).
guided_vs_plain: the metric's second half, on the caustic scene (198,936
triangles, 1024^2, 2M photon paths/iteration): relMSE against the FP64
CPU-converged oracle (tests/golden/fp64_caustic_crop.npz) of plain and guided
SPPM at equal wall time, and the guided run's time to reach the plain run's
errors, over three seeds (guide_eval; --guide-eval runs it alone).
fp64_image_errors: relMSE of plain renders of the Cornell box and of the
mixed-materials construction at 320x180 against their FP64 oracles.
--impl reference: the CPU restatement of the reference path (oracle/port,
pinned bit-exact to the reference's own outputs), compiled with the
reference's own optimisation flags, on all host cores in a child process.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, 'friendsrender-r-public_gb300'))

METRIC = 'photon paths/s; equal-time relMSE vs FP64 ref, guided vs plain SPPM, 1 GB300'
UNIT = 'photon paths/s'
PHOTONS = 1_000_000
ALPHA, RADIUS = 0.7, 0.02
WORKLOAD = ('mixed materials: 997,444 triangles (200 UV spheres + 512^2 height field), 4 surface types, '
            '1024^2 RGBA8 albedo/roughness/normal textures, 512^2 textured light, 1280x720 thin lens '
            'aperture 0.02, 1M photon paths/iteration, alpha 0.7, r0 0.02')


# Traversal work per closest-hit ray of this workload on the reference's own
# BVH (N_BVH8::findClosestElement, bvh8.h:568-641): 168 V + 40 X FP32
# operations, V internal nodes and X leaf triangle tests per ray, counted by
# the reference's harness on a 10% sample of the rays of one iteration
# (tests/golden/make_traversal_work.py -> tests/golden/traversal_work_mixed.json).
TRAVERSAL_FP32_OPS_PER_RAY = {'eye': 2336.0085393334575, 'photon': 2640.158385979652}


def fp32_peak_tflops(sm_mhz):
    """Nominal FP32 rate: SMs x 128 FP32 lanes x 2 (FMA) x SM clock."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    return sms * 128 * 2 * sm_mhz * 1e6 / 1e12


def pipelined_e2e(r, npix, steps):
    """Seconds for `steps` iterations through the C-ABI, each one's image
    copied into pinned host memory by fr_resolve_async (two buffers in turn)
    and waited for while the next iteration runs; the last wait and the
    device error check (fr_synchronize) are inside the timed region."""
    import torch
    hosts = [torch.empty((npix, 4), dtype=torch.float32, pin_memory=True) for _ in range(2)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    prev = None
    for k in range(steps):
        r.iterate(1, sync=False)
        ticket = r.resolve_async(hosts[k % 2].data_ptr())
        if prev is not None:
            r.resolve_wait(prev)  # step k-1's image is on the host
        prev = ticket
    r.resolve_wait(prev)
    r.synchronize()
    return time.perf_counter() - t0


def traversal_block(rays, eye_rays, photon_rays, trace_s, eye_q, photon_q, clocks):
    """Trace-kernel throughput: rays per second of trace-kernel time, and the
    reference's traversal work on those rays (TRAVERSAL_FP32_OPS_PER_RAY) as a
    fraction of the nominal FP32 rate at the SM clock seen while timing."""
    ops = eye_rays * TRAVERSAL_FP32_OPS_PER_RAY['eye'] + photon_rays * TRAVERSAL_FP32_OPS_PER_RAY['photon']
    mhz = clocks.get('sm_mhz') or clocks.get('sm_max_mhz') or 2070.0
    peak = fp32_peak_tflops(mhz)
    achieved = ops / trace_s / 1e12
    return {'kernel': 'k_wave_trace', 'rays_per_step': rays, 'rays_per_s': rays / trace_s,
            'tail_paths_per_step': int(eye_q[-1]) + int(photon_q[-1]),
            'reference_work': {'fp32_ops_per_ray': TRAVERSAL_FP32_OPS_PER_RAY, 'achieved_tflops': achieved,
                               'peak_tflops': peak, 'frac': achieved / peak,
                               'peak_source': 'nominal: SMs x 128 FP32 lanes x 2 x %.0f MHz' % mhz,
                               'work': '168 V + 40 X per ray on the reference BVH (bvh8.h:568-641), '
                                       'tests/golden/traversal_work_mixed.json'}}


def scene_bytes(stats):
    """Device bytes of the mixed-materials scene's data: 224-byte BVH nodes,
    48-byte leaf triangles and 64-byte shading records per triangle, three
    1024^2 RGBA8 textures and the 512^2 light texture."""
    return stats['bvh_nodes'] * 224 + stats['triangles'] * (48 + 64) + 3 * 1024 * 1024 * 4 + 512 * 512 * 4


def dist_env():
    return int(os.environ.get('RANK', 0)), int(os.environ.get('WORLD_SIZE', 1)), int(os.environ.get('LOCAL_RANK', 0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 200 ms while active."""
    Q = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,'
         'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
         'clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu):
        self.gpu = gpu
        self.p = None
        self.lines = []

    def __enter__(self):
        try:
            self.p = subprocess.Popen(['nvidia-smi', '-i', str(self.gpu), '--query-gpu=' + self.Q,
                                       '--format=csv,noheader,nounits', '-lms', '200'],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.p = None
        return self

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            f = [x.strip() for x in ln.split(',')]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == 'active':
                    reasons.add(n)
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': mx or None,
                'reasons': sorted(reasons), 'samples': len(sm)}


def measured_peaks():
    p = os.path.join(REPO, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get('hbm_gbs', 6800.0), 'measured'
    return 6800.0, 'fallback'


# The CPU side runs the oracle's timing build (oracle/port compiled with the
# reference's own optimisation flags, SPPM/SPPM/makefile: -O2 -ffast-math
# -Ofast -fopenmp; its x86-only -mavx left out) on all host threads.
CPU_FLAGS = '-O2 -ffast-math -Ofast -fopenmp (the reference makefile\'s flags without its x86-only -mavx)'


def cpu_measure(photons, warmup, steps, budget_s=None):
    """Times the oracle's timing build on the mixed-materials workload (full
    eye pass, grid, gather every iteration): warmup untimed iterations, then
    steps timed ones.  With budget_s the photons per iteration shrink so the
    whole run stays near budget_s seconds.  Runs in this process; callers run
    it in a child process, so the GPU process never maps the oracle."""
    from frsppm import scenes
    sys.path.insert(0, os.path.join(REPO, 'oracle'))
    import port_abi
    port_abi.load('timing')
    port_abi.set_threads(os.cpu_count() or 1)
    threads = port_abi.max_threads()
    scene = scenes.mixed_materials()
    if budget_s is not None:
        with port_abi.PortRenderer(scene, photons, alpha=ALPHA, radius=RADIUS, kind='timing') as r:
            t0 = time.perf_counter()
            r.iterate(1)
            per_full = time.perf_counter() - t0
        per_budget = budget_s / max(1, steps + warmup)
        if per_full > per_budget:
            photons = max(50_000, int(photons * per_budget / per_full))
    with port_abi.PortRenderer(scene, photons, alpha=ALPHA, radius=RADIUS, kind='timing') as r:
        for _ in range(warmup):
            r.iterate(1)
        t0 = time.perf_counter()
        r.iterate(steps)
        dt = time.perf_counter() - t0
    return {'value': photons * steps / dt, 'unit': UNIT, 'cores': threads, 'kind': 'port',
            'build': CPU_FLAGS, 'photons_per_step': photons, 'steps': steps, 'warmup': warmup, 'seconds': dt,
            'sample': '%d iterations of the workload (%d photon paths each, full 1280x720 eye pass, grid, gather) '
                      'after %d untimed, %d OpenMP threads, %.2f s' % (steps, photons, warmup, threads, dt)}


def cpu_child(args_json):
    """Runs cpu_measure in a child process and returns its JSON result."""
    cmd = [sys.executable, os.path.abspath(__file__), '--cpu-measure', args_json]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
    if r.returncode != 0:
        raise RuntimeError('CPU measurement failed: ' + r.stderr[-2000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_baseline():
    """The CPU baseline beside the GPU number: 4 full iterations of the same
    workload (1M paths each) after 1 untimed, in a child process."""
    return cpu_child(json.dumps({'photons': PHOTONS, 'warmup': 1, 'steps': 4}))


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    # Each step is one iteration of the workload; the photon count per step is
    # reduced when K + W full iterations would run past ~2.5 minutes.
    cb = cpu_child(json.dumps({'photons': PHOTONS, 'warmup': args.warmup, 'steps': args.steps, 'budget_s': 150.0}))
    value = cb['value']
    out = {'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
           'warmup': args.warmup, 'ms_per_step': cb['seconds'] * 1000.0 / args.steps, 'higher_is_better': True,
           'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic (seeded scene)',
           'config': {'workload': WORKLOAD, 'photons_per_step': cb['photons_per_step']}, 'impl': 'reference',
           'cpu_baseline': cb,
           'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(out))
    return 0


# Algorithmic bytes of one traced ray in k_wave_trace, the dominant kernel:
# the queue entry (4 B), the ray (origin + index of refraction, direction +
# PDF: 32 B) read and the hit record (16 B) written.  The BVH and triangle
# reads are re-reads of a resident scene, not per-ray algorithmic traffic.
TRACE_BYTES_PER_RAY = 52
TRACE_TRAFFIC_PROFILE = os.path.join(REPO, 'profiles', 'k_wave_trace_traffic_mixed_materials_1M.md')


def trace_traffic_per_launch():
    """DRAM bytes (read + write) per k_wave_trace launch that traced rays (the
    rounds of one iteration that ran, skipped rounds left out), from the
    committed ncu capture of this workload, or None."""
    try:
        for line in open(TRACE_TRAFFIC_PROFILE):
            if line.startswith('bytes_per_nonempty_launch:'):
                return float(line.split(':', 1)[1])
    except OSError:
        pass
    return None


# ---- guided vs plain SPPM on the caustic scene at equal wall time
CAUSTIC_PHOTONS = 2_000_000
CAUSTIC_ALPHA, CAUSTIC_RADIUS = 0.7, 0.01
CAUSTIC_WORKLOAD = ('caustic box: 198,936 triangles (50 GGX-dielectric spheres, IOR 1.5, roughness 0.02, on a '
                    'diffuse floor) in a diffuse box lit through a 0.1x0.1 slit in its top by a 1x1 textured area '
                    'light, 1024^2 pinhole, 2M photon paths/iteration, alpha 0.7, r0 0.01')
REL_MSE_EPS = 1e-2


def _linear(img):
    """fr_resolve's pixels (radiance to the power 1/1.2) back to radiance."""
    return img[:, :3].astype('float64') ** 1.2


def rel_mse(img, ref):
    """Mean over pixels and channels of (x - r)^2 / (r^2 + 1e-2), radiance."""
    a, b = _linear(img), _linear(ref)
    return float(((a - b) ** 2 / (b * b + REL_MSE_EPS)).mean())


GOLDEN = os.path.join(REPO, 'tests', 'golden')


def fp64_oracle(name):
    """A committed FP64 CPU-converged oracle image (tests/golden/fp64_<name>.npz,
    made by tests/golden/make_fp64_oracle.py): linear radiance (h, w, 3), the
    window of the frame it covers (x0, y0, x1, y1; zeros for the whole frame)
    and the photon paths it holds."""
    d = np.load(os.path.join(GOLDEN, 'fp64_%s.npz' % name))
    return d['radiance'].astype(np.float64), tuple(int(v) for v in d['window']), int(d['photon_paths'])


def rel_mse_linear(img, width, ref, window):
    """relMSE of a resolved image (fr_resolve: radiance^(1/1.2)) against linear
    reference radiance over the reference's window of the frame, both scaled
    so that the reference's mean is 1 (the 1e-2 in the denominator is then
    relative to the image's own brightness)."""
    a = _linear(img).reshape(-1, width, 3)
    if window != (0, 0, 0, 0):
        x0, y0, x1, y1 = window
        a = a[y0:y1, x0:x1]
    k = 1.0 / ref.mean()
    a, b = a * k, ref * k
    return float(((a - b) ** 2 / (b * b + REL_MSE_EPS)).mean())


GUIDE_SEEDS = (1, 2, 3)


def guide_eval(plain_iters=128, photons=CAUSTIC_PHOTONS, scene=None, log=None, eager=False, seeds=GUIDE_SEEDS):
    """Plain and guided SPPM on the caustic box against the FP64 CPU-converged
    oracle (the 256^2 window in the middle of the 1024^2 frame), all resolved
    with the standard estimate tau / (pi R^2 photons emitted) and with
    degenerate paths ended.  For each seed (the guide's initial weights, and
    both runs' random streams moved by fr_seek), the plain run's error after
    1/4, 1/2 and all of plain_iters iterations are the targets; the guided
    run's wall time to first reach each (checked at iteration marks 12.5%
    apart) and its error at the plain run's final wall time are reported, with
    the minimum and median over the seeds.  Wall time is fr_iterate +
    fr_synchronize, the guide's training included; the resolves at the marks
    are not timed.  eager: iterations launched directly (stage profiler on)
    instead of as the captured graph, whose conditional nodes ncu cannot
    profile into; for kernel profiles only."""
    from frsppm import abi, scenes
    scene = scene or scenes.caustic_box()
    ref, window, ref_paths = fp64_oracle('caustic_crop')
    width = scene['camera']['width']
    kw = dict(alpha=CAUSTIC_ALPHA, radius=CAUSTIC_RADIUS,
              flags=abi.FLAG_STANDARD_RESOLVE | abi.FLAG_END_DEGENERATE_PATHS)
    max_run = 4 * plain_iters
    marks, m = [], 1.0
    while int(m) < plain_iters:
        if not marks or int(m) > marks[-1]:
            marks.append(int(m))
        m *= 1.125
    marks.append(plain_iters)

    def run(guided, seed, stop):
        curve = []
        extra = dict(guide=True, guide_seed=seed) if guided else {}
        with abi.Renderer(scene, photons, **kw, **extra) as r:
            r.seek(1000 * seed)
            if eager:
                r.profile(True, max_iterations=max_run + len(marks) + 1)
            r.synchronize()
            t, done, k = 0.0, 0, 0
            while True:
                target = marks[k] if k < len(marks) else int(done * 1.125) + 1
                t1 = time.perf_counter()
                r.iterate(target - done)
                t += time.perf_counter() - t1
                done = target
                curve.append((done, t, rel_mse_linear(r.resolve(), width, ref, window)))
                if log:
                    log('%s seed %d: %d iterations %.3f s relMSE %.5f' % ('guided' if guided else 'plain', seed,
                                                                          *curve[-1]))
                k += 1
                if stop(done, t):
                    return curve

    per_seed = []
    for seed in seeds:
        plain = run(False, seed, lambda n, t: n >= plain_iters)
        t_plain = plain[-1][1]
        guided = run(True, seed, lambda n, t: t >= 1.02 * t_plain or n >= max_run)
        targets = {}
        for frac in (4, 2, 1):
            n_t = plain_iters // frac
            e_t, t_t = next((e, t) for n, t, e in plain if n >= n_t)
            reach = next(((n, t) for n, t, e in guided if e <= e_t), None)
            targets['plain_%d_iterations' % n_t] = {
                'rel_mse': e_t, 'plain_wall_s': t_t,
                'guided_iterations': reach[0] if reach else None, 'guided_wall_s': reach[1] if reach else None,
                'speedup': (t_t / reach[1]) if reach else None}
        at_equal = [e for n, t, e in guided if t <= t_plain]
        per_seed.append({
            'seed': seed,
            'plain': {'iterations': plain_iters, 'wall_s': t_plain, 'rel_mse': plain[-1][2],
                      'ms_per_iteration': 1e3 * t_plain / plain_iters},
            'guided': {'rel_mse_at_equal_time': at_equal[-1] if at_equal else None,
                       'ms_per_iteration': 1e3 * guided[-1][1] / guided[-1][0]},
            'time_to_target': targets,
            'curves': {'plain': [[n, round(t, 4), round(e, 6)] for n, t, e in plain],
                       'guided': [[n, round(t, 4), round(e, 6)] for n, t, e in guided]}})

    def stat(key):
        v = [p['time_to_target'][key]['speedup'] for p in per_seed]
        ok = [x for x in v if x is not None]
        return {'min': min(ok) if len(ok) == len(v) else None, 'median': float(np.median(ok)) if ok else None,
                'per_seed': v}
    keys = list(per_seed[0]['time_to_target'])
    return {
        'workload': CAUSTIC_WORKLOAD,
        'reference': ('FP64 CPU-converged oracle (oracle/port in double, standard resolve, degenerate paths '
                      'ended, own random streams): the %dx%d window at (%d, %d), %d photon paths'
                      % (window[2] - window[0], window[3] - window[1], window[0], window[1], ref_paths)),
        'rel_mse': ('mean of (x - ref)^2 / (ref^2 + %g) over the window\'s pixels and RGB, linear radiance '
                    'scaled so that the reference\'s mean is 1' % REL_MSE_EPS),
        'seeds': list(seeds),
        'time_to_plain_error_speedup': {k: stat(k) for k in keys},
        'rel_mse_at_equal_time': {'plain': [p['plain']['rel_mse'] for p in per_seed],
                                  'guided': [p['guided']['rel_mse_at_equal_time'] for p in per_seed]},
        'per_seed': per_seed,
    }


def fp64_image_errors():
    """relMSE of plain GPU renders against their FP64 CPU-converged oracles
    (standard resolve): the Cornell box (256^2, 100k paths, its 16 iterations
    and more) and the mixed-materials construction at 320x180 (1M paths, its 64
    iterations)."""
    from frsppm import abi, scenes
    out = {}
    cases = (('cornell', lambda: scenes.cornell_box(), 100_000, 0.7, 0.02, (16, 64, 256)),
             ('mixed_small', lambda: scenes.mixed_materials(width=320, height=180), 1_000_000, 0.7, 0.02, (16, 64)))
    for name, factory, photons, alpha, radius, marks in cases:
        ref, window, ref_paths = fp64_oracle(name)
        scene = factory()
        width = scene['camera']['width']
        errs = {}
        with abi.Renderer(scene, photons, alpha=alpha, radius=radius, flags=abi.FLAG_STANDARD_RESOLVE) as r:
            done = 0
            for m in marks:
                r.iterate(m - done)
                done = m
                errs[str(m)] = rel_mse_linear(r.resolve(), width, ref, window)
        out[name] = {'photons_per_iteration': photons, 'rel_mse_by_iterations': errs,
                     'oracle_photon_paths': ref_paths}
    return out


LARGE_PHOTONS = 8_000_000
LARGE_WORKLOAD = ('large scene: 20,000,004 triangles (400 copies of a 50,000-triangle seeded displaced geodesic '
                  'sphere, flattened), 16 materials of all four surface types, 4096^2 RGBA8 albedo/roughness/normal '
                  'textures, 512^2 textured light, 3840x2160 thin lens aperture 0.02, 8M photon paths/iteration, '
                  'learned guide on, alpha 0.7, r0 0.02')


def bvh_builder(args):
    from frsppm import abi
    return abi.BVH_DEVICE_LBVH if args.bvh == 'lbvh' else abi.BVH_HOST_SAH


def run_large(args):
    """The large-scene workload: photon paths/s of guided SPPM iterations
    (graph replays, CUDA events on the renderer's stream; the working set is
    far larger than L2), and the same through the C-ABI with the image read
    back every step."""
    import torch
    from frsppm import abi, scenes
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    scene = scenes.large_scene()
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    r = abi.Renderer(scene, LARGE_PHOTONS, alpha=ALPHA, radius=RADIUS, guide=True,
                     flags=abi.FLAG_END_DEGENERATE_PATHS, bvh_builder=bvh_builder(args))
    setup_s = time.perf_counter() - t0
    stats = r.stats()
    npix = r.width * r.height
    stream = torch.cuda.ExternalStream(r.stream())
    W = max(3, args.warmup)
    r.iterate(W)
    l0 = r.profile_read()[2]
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        a.record(stream)
        r.iterate(args.steps, sync=False)
        b.record(stream)
        stream.synchronize()
    ms = a.elapsed_time(b)
    launches = r.profile_read()[2] - l0
    e2e_s = pipelined_e2e(r, npix, args.steps)
    eye_q, photon_q = r.wave_counts()
    r.close()
    out = {'metric': METRIC, 'value': LARGE_PHOTONS * args.steps / (ms / 1000.0), 'unit': UNIT, 'n_gpus': 1,
           'steps': args.steps, 'warmup': W, 'ms_per_step': ms / args.steps, 'higher_is_better': True,
           'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic (seeded scene)',
           'config': {'workload': LARGE_WORKLOAD, 'photons_per_step': LARGE_PHOTONS, 'pixels': npix, 'bvh': args.bvh,
                      'triangles': stats['triangles'], 'bvh_nodes': stats['bvh_nodes'],
                      'l2': 'working set far above L2 (photon slots alone 12.3 GB)'},
           'hitpoint_updates_per_s': npix * args.steps / (ms / 1000.0),
           'e2e': {'value': LARGE_PHOTONS * args.steps / e2e_s, 'unit': UNIT, 'h2d_bytes_per_step': 0,
                   'd2h_bytes_per_step': npix * 16, 'scene_generation_s': gen_s, 'setup_s': setup_s,
                   'device_bytes': int(stats['device_bytes'])},
           'gpu_launches': launches, 'clocks': clk.summary(),
           'tail_paths_per_step': [int(eye_q[-1]), int(photon_q[-1])]}
    print(json.dumps(out))
    return 0


BATCH_WORKLOAD = ('batched uneven SPPM: 64 seeded scenes of the mixed-materials construction, triangles '
                  'log-uniform over 10k-2M (30.5M in all), resolutions uniform over 128^2/256^2/512^2/1024^2, '
                  '50k-1M photon paths/iteration each (33.8M in all), 256^2 textures, alpha 0.7, r0 0.02; '
                  'each context autotuned by fr_autotune, then all advanced by one batch graph (fr_batch_create: '
                  'one graph launch per step for all 64 scenes)')


def run_batch(args):
    """The batched workload: one step is one iteration of every scene
    (fr_iterate_batch).  value = photon paths of all scenes / wall time of the
    batch steps; the same scenes iterated one after another (each context's
    graph-replay time, CUDA events) are reported beside it."""
    # More hardware queues for the contexts' streams (read at context creation).
    os.environ.setdefault('CUDA_DEVICE_MAX_CONNECTIONS', '32')
    import multiprocessing
    from concurrent.futures import ProcessPoolExecutor
    from frsppm import scenes
    specs = scenes.batch_specs()
    t0 = time.perf_counter()
    with ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1),
                             mp_context=multiprocessing.get_context('spawn')) as ex:
        scene_list = list(ex.map(scenes.batch_scene, specs))
    gen_s = time.perf_counter() - t0
    import torch
    from frsppm import abi
    torch.cuda.set_device(dist_env()[2])
    t0 = time.perf_counter()
    rs = [abi.Renderer(sc, sp['photons'], alpha=ALPHA, radius=RADIUS, bvh_builder=bvh_builder(args))
          for sc, sp in zip(scene_list, specs)]
    setup_s = time.perf_counter() - t0
    tuned = [r.autotune(1) if not args.no_autotune else None for r in rs]
    # One after another: each context's graph replays alone.
    seq_ms = 0.0
    for r in rs:
        s = torch.cuda.ExternalStream(r.stream())
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r.iterate(1)
        a.record(s)
        r.iterate(2, sync=False)
        b.record(s)
        r.synchronize()
        seq_ms += a.elapsed_time(b) / 2
    W = max(3, args.warmup)
    # The same steps with one graph per context (fr_iterate_batch), for
    # comparison with the batch graph below.
    abi.iterate_batch(rs, W)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    abi.iterate_batch(rs, args.steps)
    per_context_dt = time.perf_counter() - t0
    # One graph holding an iteration of every scene (fr_batch_create): one
    # graph launch per step.
    batch = abi.Batch(rs)
    batch.iterate(W)
    torch.cuda.synchronize()
    l0 = sum(r.profile_read()[2] for r in rs)
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        batch.iterate(args.steps)
        dt = time.perf_counter() - t0
    launches = sum(r.profile_read()[2] for r in rs) - l0
    # End to end: every step, every scene's image copied into pinned host
    # memory (fr_resolve_async, two buffers per scene in turn) and waited for
    # while the next step runs.
    hosts = [[torch.empty((r.width * r.height, 4), dtype=torch.float32, pin_memory=True) for _ in range(2)]
             for r in rs]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    prev = None
    for k in range(args.steps):
        batch.iterate(1, sync=False)
        tickets = [r.resolve_async(h[k % 2].data_ptr()) for r, h in zip(rs, hosts)]
        if prev is not None:
            for r, t in zip(rs, prev):
                r.resolve_wait(t)
        prev = tickets
    for r, t in zip(rs, prev):
        r.resolve_wait(t)
        r.synchronize()
    e2e_dt = time.perf_counter() - t0
    photons = sum(sp['photons'] for sp in specs)
    pixels = sum(r.width * r.height for r in rs)
    dev = sum(r.stats()['device_bytes'] for r in rs)
    tris = sum(len(sc['pos']) for sc in scene_list)
    batch.close()
    for r in rs:
        r.close()
    hist = {}
    for t in tuned:
        hist[str(t)] = hist.get(str(t), 0) + 1
    out = {'metric': METRIC, 'value': photons * args.steps / dt, 'unit': UNIT, 'n_gpus': 1, 'steps': args.steps,
           'warmup': W, 'ms_per_step': 1e3 * dt / args.steps, 'higher_is_better': True, 'scaling': 'weak',
           'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic (seeded scenes)',
           'config': {'workload': BATCH_WORKLOAD, 'scenes': len(rs), 'triangles': tris, 'bvh': args.bvh,
                      'photons_per_step': photons, 'pixels': pixels,
                      'l2': 'working set far above L2 (64 contexts, %.1f GB)' % (dev / 1e9)},
           'hitpoint_updates_per_s': pixels * args.steps / dt,
           'sequential': {'ms_per_step': seq_ms, 'value': photons / (seq_ms / 1e3),
                          'note': 'sum over the scenes of one graph replay alone (CUDA events)'},
           'batch_speedup': seq_ms / (1e3 * dt / args.steps),
           'graph_launches_per_step': 1,
           'per_context_graphs': {'ms_per_step': 1e3 * per_context_dt / args.steps,
                                  'value': photons * args.steps / per_context_dt,
                                  'note': 'fr_iterate_batch: one graph launch per scene and step'},
           'autotune': {'photon_tail_min_chosen': hist},
           'setup': {'scene_generation_s': gen_s, 'contexts_s': setup_s, 'device_bytes': int(dev)},
           'e2e': {'value': photons * args.steps / e2e_dt, 'unit': UNIT, 'h2d_bytes_per_step': 0,
                   'd2h_bytes_per_step': pixels * 16},
           'gpu_launches': launches, 'clocks': clk.summary()}
    print(json.dumps(out))
    return 0


# Bytes one N/tau/R update (k_update) must move: read M 4, the flux sums as
# float4 16 (fr_update_dev's layout), N 4, tau 24 (FP64 x 3), R 4, NumGather 4;
# write tau 24, R 4, N 4, NumGather 4.
UPDATE_BYTES_PER_PIXEL = 92


def run_update(args):
    """The N/tau/R update alone (fr_update_dev) over a 3840x2160 pixel state,
    every pixel with photons: hitpoint updates/s and the kernel's achieved
    HBM bandwidth (the working set, 8.3M x 92 B, is far above L2)."""
    import torch
    from frsppm import abi, scenes
    torch.cuda.set_device(dist_env()[2])
    r = abi.Renderer(scenes.cornell_box(width=3840, height=2160), 1000, alpha=ALPHA, radius=RADIUS)
    npix = r.width * r.height
    gen = torch.Generator(device='cuda')
    gen.manual_seed(1)
    m = torch.randint(1, 8, (npix,), dtype=torch.int32, device='cuda', generator=gen)
    phi = torch.rand((npix, 4), device='cuda', generator=gen)
    torch.cuda.synchronize()
    W = max(3, args.warmup)
    for _ in range(W):
        r.update_dev(m.data_ptr(), phi.data_ptr(), sync=False)
    stream = torch.cuda.ExternalStream(r.stream())
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    r.synchronize()
    with ClockSampler(dist_env()[2]) as clk:
        for a, b in evs:
            a.record(stream)
            r.update_dev(m.data_ptr(), phi.data_ptr(), sync=False)
            b.record(stream)
        r.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
    r.close()
    peak, kind = measured_peaks()
    achieved = UPDATE_BYTES_PER_PIXEL * npix / (ms / 1e3) / 1e9
    out = {'metric': 'hitpoint updates/s (N/tau/R update alone)', 'value': npix / (ms / 1e3),
           'unit': 'hitpoint updates/s', 'n_gpus': 1, 'steps': args.steps, 'warmup': W, 'ms_per_step': ms,
           'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
           'data': 'synthetic (random per-pixel counts 1-7 and flux sums)',
           'config': {'workload': 'fr_update_dev over 3840x2160 = 8,294,400 pixels, every pixel updated',
                      'l2': 'inputs larger than L2 (763 MB per step)'},
           'roofline': {'bound': 'hbm', 'kernel': 'k_update', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                        'frac': achieved / peak, 'traffic': None, 'peak_source': kind,
                        'algorithmic_bytes_per_launch': UPDATE_BYTES_PER_PIXEL * npix},
           'gpu_launches': args.steps, 'clocks': clk.summary()}
    print(json.dumps(out))
    return 0


def run_ncu_pass(args):
    """--ncu-pass: args.steps iterations of the mixed-materials workload with
    the stage profiler on from the first one, so that every kernel is a direct
    launch in issue order (per iteration: the photon pass, then the eye pass,
    the grid and the gather), each iteration after a 256 MB L2 flush."""
    import torch
    from frsppm import abi, scenes
    r = abi.Renderer(scenes.mixed_materials(), args.photons, alpha=ALPHA, radius=RADIUS)
    r.profile(True, max_iterations=max(1, args.steps))
    stream = torch.cuda.ExternalStream(r.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device='cuda')
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        r.iterate(1)
    stage_ms, _, launches = r.profile_read()
    r.close()
    print(json.dumps({'ncu_pass': True, 'photons': args.photons, 'steps': args.steps, 'launches': launches,
                      'stage_ms': stage_ms}))
    return 0


def other_workloads():
    """The batched uneven scenes (64 contexts, fr_iterate_batch) and the large
    scene (20M triangles, 3840x2160, 8M paths, guide on), each measured by its
    own --workload run in a child process (so each starts with the GPU to
    itself); their JSON lines, shortened."""
    out = {}
    for name, extra in (('batch', ['--steps', '3', '--warmup', '3']), ('large', ['--steps', '5', '--warmup', '3'])):
        cmd = [sys.executable, os.path.abspath(__file__), '--workload', name] + extra
        t0 = time.perf_counter()
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
            line = json.loads(r.stdout.strip().splitlines()[-1]) if r.returncode == 0 else None
        except (subprocess.TimeoutExpired, ValueError, IndexError):
            line = None
        if line is None:
            out[name] = {'unavailable': 'the --workload %s run failed' % name}
            continue
        keep = ('value', 'unit', 'ms_per_step', 'steps', 'warmup', 'hitpoint_updates_per_s', 'e2e', 'gpu_launches',
                'clocks', 'batch_speedup', 'sequential', 'setup', 'graph_launches_per_step', 'per_context_graphs')
        out[name] = {k: line[k] for k in keep if k in line}
        out[name]['workload'] = line['config']['workload']
        out[name]['run_s'] = time.perf_counter() - t0
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=None,
                    help='timed steps (default: 200 for the mixed-materials and update workloads, whose steps '
                         'take milliseconds, so that the clock sampler sees the timed region; 10 otherwise)')
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--photons', type=int, default=PHOTONS)
    ap.add_argument('--guide-eval', action='store_true', help='only the guided-vs-plain caustic comparison')
    ap.add_argument('--no-guide-eval', action='store_true')
    ap.add_argument('--guide-plain-iters', type=int, default=128)
    ap.add_argument('--guide-photons', type=int, default=CAUSTIC_PHOTONS)
    ap.add_argument('--eager', action='store_true', help='guide eval: direct launches (for ncu)')
    ap.add_argument('--workload', default='mixed', choices=['mixed', 'large', 'batch', 'update'],
                    help='large: the 20M-triangle scene; batch: 64 uneven scenes; update: the N/tau/R update '
                         'alone (each its own JSON line)')
    ap.add_argument('--no-autotune', action='store_true')
    ap.add_argument('--bvh', default='sah', choices=['sah', 'lbvh'],
                    help='scene BVH: host binned SAH (default) or the device LBVH build')
    ap.add_argument('--cpu-measure', default=None, help=argparse.SUPPRESS)
    ap.add_argument('--ncu-pass', action='store_true',
                    help='only --steps iterations of the mixed-materials workload with the stage profiler on (every '
                         'kernel a direct launch, none inside a graph), each after a 256 MB L2 flush: the pass '
                         'that kernel-profiler captures select launches from')
    ap.add_argument('--no-other-workloads', action='store_true',
                    help='skip the batched-scenes and large-scene lines embedded in the default line')
    args = ap.parse_args()
    if args.cpu_measure is not None:
        print(json.dumps(cpu_measure(**json.loads(args.cpu_measure))))
        return 0
    if args.steps is None:
        args.steps = 200 if args.impl == 'ours' and args.workload in ('mixed', 'update') else 10
    if args.impl == 'reference':
        return run_reference(args)
    if args.ncu_pass:
        return run_ncu_pass(args)
    if args.workload == 'large':
        return run_large(args)
    if args.workload == 'batch':
        return run_batch(args)
    if args.workload == 'update':
        return run_update(args)
    if args.guide_eval:
        out = guide_eval(args.guide_plain_iters, args.guide_photons,
                         log=lambda s: print(s, file=sys.stderr, flush=True), eager=args.eager)
        print(json.dumps(out))
        return 0

    import numpy as np
    import torch
    from frsppm import abi, scenes

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl')
    W = max(3, args.warmup)
    scene = scenes.mixed_materials()
    t0 = time.perf_counter()
    r = abi.Renderer(scene, args.photons, alpha=ALPHA, radius=RADIUS, bvh_builder=bvh_builder(args))
    setup_s = time.perf_counter() - t0
    stats = r.stats()
    npix = r.width * r.height
    stream = torch.cuda.ExternalStream(r.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device='cuda')
    r.iterate(W)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- device-timed region: the steps back to back, as a render loop runs
    # them (an iteration's gather overlaps the next iteration's photon pass),
    # in one pair of events on the main stream; the window closes after the
    # main stream has waited for the last gather (fr_stream joins the pixel
    # stream).  No flush between steps: the inputs are larger than L2.
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = r.profile_read()[2]
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        a.record(stream)
        for k in range(args.steps):
            r.iterate(1, sync=False)
        r.stream()
        b.record(stream)
        stream.synchronize()
    torch.cuda.synchronize()
    barrier()
    l1 = r.profile_read()[2]
    total_ms = a.elapsed_time(b)
    if world > 1:
        t = torch.tensor([total_ms], device='cuda')
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    launches = l1 - l0

    # ---- the same steps one at a time, L2 flushed (256 MB write) before each,
    # each step's window closed after its own gather (no overlap across steps)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            evs[k][0].record(stream)
        r.iterate(1, sync=False)
        r.stream()
        evs[k][1].record(stream)
    stream.synchronize()
    flushed_ms = sum(x.elapsed_time(y) for x, y in evs) / args.steps

    # ---- the same steps again with the stage profiler's CUDA events (stage and
    # trace-kernel durations for the roofline; launched directly, not as a graph)
    r.profile(True, max_iterations=args.steps)
    torch.cuda.synchronize()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        r.iterate(1, sync=False)
    stream.synchronize()
    stage_ms, stage_n, _ = r.profile_read()
    r.profile(False)

    # ---- rays traced and photons stored in the last timed iteration
    eye_q, photon_q = r.wave_counts()
    eye_rays, photon_rays = int(eye_q[:-1].sum()), int(photon_q[:-1].sum())
    rays = eye_rays + photon_rays
    counts = np.empty(r.photons, np.uint32)
    abi._check(abi._lib.fr_read_photon_slots(r.h, None, None, None, abi._ptr(counts)), 'fr_read_photon_slots')
    stored = int(counts.sum())
    hits = int((r.read_hitpoints()['type'] == 1).sum())

    # ---- end to end through the C-ABI with pinned host result buffers: every
    # step's image is copied to the host (fr_resolve_async, two buffers in
    # turn) and waited for while the next step runs; the last one and the
    # device error check close the timed region.
    barrier()
    e2e_s = pipelined_e2e(r, npix, args.steps)
    if world > 1:
        t = torch.tensor([e2e_s], device='cuda')
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    r.close()

    if rank != 0:
        return 0
    value = world * args.photons * args.steps / (total_ms / 1000.0)
    per = {k: stage_ms[k] / args.steps for k in stage_ms}
    peak, peak_kind = measured_peaks()
    # Trace launches that traced rays (rounds that ran; the skipped rounds'
    # launches return at once and their few microseconds stay in trace_s).
    trace_launches = int((eye_q[:-1] > 0).sum() + (photon_q[:-1] > 0).sum())
    trace_s = (stage_ms['eye_trace'] + stage_ms['photon_trace']) / 1000.0 / args.steps
    bytes_per_step = rays * TRACE_BYTES_PER_RAY
    bytes_per_launch = bytes_per_step / trace_launches
    achieved = bytes_per_step / trace_s / 1e9
    clocks = clk.summary()
    out = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps, 'warmup': W,
        'ms_per_step': total_ms / args.steps, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32', 'data': 'synthetic (seeded scene, random-init textures)',
        'config': {'workload': WORKLOAD, 'photons_per_step': args.photons, 'pixels': npix, 'bvh': args.bvh,
                   'triangles': stats['triangles'], 'bvh_nodes': stats['bvh_nodes'],
                   'l2': 'inputs larger than L2: scene data %.0f MB (BVH nodes, triangles, shading records, '
                         'textures), %.1f GB of device state, about 0.6 GB of it touched per step; steps back to '
                         'back' % (scene_bytes(stats) / 1e6, stats['device_bytes'] / 1e9),
                   'parallelism': 'replicas' if world > 1 else 'single GPU'},
        'flushed_steps': {'ms_per_step': flushed_ms, 'value': world * args.photons / (flushed_ms / 1000.0),
                          'note': 'each step alone: L2 flushed (256 MB write) before it, its window closed after '
                                  'its own gather, so no step overlaps the next'},
        'hitpoint_updates_per_s': world * npix * args.steps / (total_ms / 1000.0),
        'stage_ms_per_step': per,
        'roofline': {'bound': 'hbm', 'kernel': 'k_wave_trace', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                     'frac': achieved / peak, 'traffic': trace_traffic_per_launch(), 'peak_source': peak_kind,
                     'algorithmic_bytes_per_launch': bytes_per_launch, 'launches_per_step': trace_launches,
                     'per': 'launch that traced rays (traffic and algorithmic bytes alike)',
                     'note': 'latency-bound BVH traversal; eye and photon launches overlap in time, and the '
                             'eye rounds run on half the resident grid (leaving the photon pass, the critical '
                             'path, the rest), which lengthens their launches'},
        'traversal': traversal_block(rays, eye_rays, photon_rays, trace_s, eye_q, photon_q, clocks),
        'e2e': {'value': world * args.photons * args.steps / e2e_s, 'unit': UNIT, 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': npix * 16, 'setup_s': setup_s,
                'device_bytes': int(stats['device_bytes'])},
        'gpu_launches': launches,
        'clocks': clocks,
        'photons_stored_last_step': stored, 'hitpoints_last_step': hits,
    }
    if world == 1 and not args.no_guide_eval:
        # equal-time relMSE, guided vs plain SPPM (caustic scene; not the timed workload)
        try:
            out['guided_vs_plain'] = guide_eval(args.guide_plain_iters, args.guide_photons)
            out['fp64_image_errors'] = fp64_image_errors()
        except OSError as e:  # an FP64 oracle image is missing
            out['guided_vs_plain'] = {'unavailable': str(e)}
    if world == 1 and not args.no_cpu_baseline:
        out['cpu_baseline'] = cpu_baseline()
    if world == 1 and not args.no_other_workloads:
        out['other_workloads'] = other_workloads()
    print(json.dumps(out))
    return 0


if __name__ == '__main__':
    sys.exit(main())
