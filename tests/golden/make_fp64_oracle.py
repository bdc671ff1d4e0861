"""Makes the FP64 CPU-converged oracle images (tests/golden/fp64_*.npz).

Each is the oracle's SPPM estimator (oracle/port, built with
FR_PORT_REAL=double: every float of the reference's path evaluated in double,
tau in double) run for many iterations on the CPU, resolved with the standard
estimate tau / (pi R^2 photons emitted) in linear radiance (pi = 3.14159, the
reference's constant).  Paths that turn degenerate (a NaN BSDF value or pdf,
a zero pdf, or an overflowed flux or PDF product) end, as with
FR_FLAG_END_DEGENERATE_PATHS.  The random streams use a second Philox key word
of their own (0x4F524331), so they share nothing with any render they judge.

Images:
  caustic_crop  the caustic box (1024^2 pinhole, 2M photon paths per
                iteration, alpha 0.7, r0 0.01), the 256^2 window at
                (384, 384) in the middle of the frame, where the light through
                the slit and the glass spheres' caustics land;
  cornell       the Cornell box (256^2, 100k paths per iteration, alpha 0.7,
                r0 0.02), whole frame;
  mixed_small   the mixed-materials scene's construction (1M triangles,
                textures, thin lens) at 320x180, 1M paths per iteration,
                alpha 0.7, r0 0.02.

Usage: python tests/golden/make_fp64_oracle.py NAME ITERATIONS [THREADS]
The image is rewritten every 32 iterations, so a run can be stopped early;
the file records the iterations and photon paths it holds.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, 'friendsrender-r-public_gb300'))
sys.path.insert(0, os.path.join(REPO, 'oracle'))

STREAM_KEY = 0x4F524331
PI_REF = 3.14159


def _cases():
    from frsppm import scenes
    return {
        'caustic_crop': dict(scene=lambda: scenes.caustic_box(), photons=2_000_000, alpha=0.7, radius=0.01,
                             window=(384, 384, 640, 640)),
        'cornell': dict(scene=lambda: scenes.cornell_box(), photons=100_000, alpha=0.7, radius=0.02, window=None),
        'mixed_small': dict(scene=lambda: scenes.mixed_materials(width=320, height=180), photons=1_000_000,
                            alpha=0.7, radius=0.02, window=None),
    }


def standard_radiance(state, photons_total, width, window):
    """tau / (pi R^2 photons emitted) per pixel, (h, w, 3) float64."""
    tau = state['tau'].astype(np.float64)
    r = state['r'].astype(np.float64)
    L = tau / (photons_total * PI_REF * r * r)[:, None]
    height = len(r) // width
    L = L.reshape(height, width, 3)
    if window:
        x0, y0, x1, y1 = window
        L = L[y0:y1, x0:x1]
    return L


def main():
    import port_abi
    name, iters = sys.argv[1], int(sys.argv[2])
    threads = int(sys.argv[3]) if len(sys.argv) > 3 else (os.cpu_count() or 1)
    case = _cases()[name]
    port_abi.set_threads(threads)
    scene = case['scene']()
    width = scene['camera']['width']
    out = os.path.join(HERE, 'fp64_%s.npz' % name)
    t0 = time.time()
    with port_abi.PortRenderer(scene, case['photons'], alpha=case['alpha'], radius=case['radius'], kind='f64') as r:
        lib = r.lib
        lib.port_set_stream_key(r.h, STREAM_KEY)
        lib.port_set_end_degenerate(r.h, 1)
        if case['window']:
            lib.port_set_window(r.h, *case['window'])
        done = 0
        while done < iters:
            n = min(32, iters - done)
            r.iterate(n)
            done += n
            L = standard_radiance(r.read_state(), float(case['photons']) * done, width, case['window'])
            np.savez_compressed(out + '.tmp.npz', radiance=L.astype(np.float32), iterations=done,
                                photon_paths=case['photons'] * done, window=np.asarray(case['window'] or (0, 0, 0, 0)),
                                photons_per_iteration=case['photons'], alpha=case['alpha'], radius=case['radius'],
                                stream_key=STREAM_KEY, seconds=time.time() - t0, threads=threads)
            os.replace(out + '.tmp.npz', out)
            print('%s: %d iterations, %.0f s, mean radiance %.6g, non-finite %d' % (
                name, done, time.time() - t0, float(np.nanmean(L)), int((~np.isfinite(L)).sum())), flush=True)


if __name__ == '__main__':
    main()
