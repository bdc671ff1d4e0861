"""fr_radius_count_noalloc: the radius count for callers that cannot let the
library allocate device memory (cudaMalloc/cudaFree synchronize the device;
applications with a fixed device-memory pool cannot have a library allocate
on its own).  Its results must equal fr_radius_query's on the same inputs,
call after call, although every call reuses the same fixed scratch arrays.

Kept in a file of its own that pytest collects last."""
import ctypes

import numpy as np
import pytest

from conftest import GOLDEN_SCENES

pytestmark = pytest.mark.gpu


def _inputs(seed, nh, np_):
    rng = np.random.Generator(np.random.PCG64(seed))
    ph = rng.uniform(-1, 1, (np_, 3)).astype(np.float32)
    ph[:, 1] = rng.choice([-0.5, 0.0, 0.5], np_)          # photons on planes, as SPPM deposits them
    hp = rng.uniform(-1, 1, (nh, 3)).astype(np.float32)
    hp[:, 1] = rng.choice([-0.5, 0.0, 0.5], nh)
    R = rng.uniform(0.005, 0.05, nh).astype(np.float32)
    return hp, R, ph


def test_noalloc_count_matches_radius_query_on_consecutive_calls():
    import torch
    from frsppm import abi
    lib = abi.load()
    cell = 0.04
    with abi.Renderer(GOLDEN_SCENES['cornell32'](), 16) as r:
        for call, (seed, nh, np_) in enumerate([(21, 20_000, 200_000), (22, 7_000, 150_000)]):
            hp, R, ph = _inputs(seed, nh, np_)
            want, _ = r.radius_query(hp, R, ph, cell)
            hp_dev = torch.from_numpy(np.concatenate([hp, R[:, None]], 1)).cuda()
            ph_dev = torch.from_numpy(ph).cuda()
            out = torch.full((nh,), -1, dtype=torch.int32, device='cuda')
            stream = torch.cuda.current_stream().cuda_stream
            rc = lib.fr_radius_count_noalloc(ctypes.c_void_p(hp_dev.data_ptr()), nh, ctypes.c_void_p(ph_dev.data_ptr()),
                                             np_, ctypes.c_float(cell), ctypes.c_void_p(out.data_ptr()),
                                             ctypes.c_void_p(stream))
            assert rc == 0, lib.fr_last_error()
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert want.sum() > 0
            np.testing.assert_array_equal(got, want, err_msg='call %d' % call)


def test_noalloc_rejects_more_photons_than_its_scratch():
    import torch
    from frsppm import abi
    lib = abi.load()
    limit = 262144  # FR_NOALLOC_MAX_PHOTONS
    hp_dev = torch.zeros((4, 4), dtype=torch.float32, device='cuda')
    ph_dev = torch.zeros((limit + 1, 3), dtype=torch.float32, device='cuda')
    out = torch.zeros(4, dtype=torch.int32, device='cuda')
    rc = lib.fr_radius_count_noalloc(ctypes.c_void_p(hp_dev.data_ptr()), 4, ctypes.c_void_p(ph_dev.data_ptr()),
                                     limit + 1, ctypes.c_float(0.1), ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 1  # FR_ERR_INVALID
    assert b'exceed' in lib.fr_last_error()


def test_noalloc_marks_unbounded_balls_and_checks_alignment():
    """Device inputs cannot be checked on the host without waiting for them:
    a hitpoint whose radius is not finite, or whose ball is more than 128
    cells wide, gets the count -1 and the others their counts.  A hitpoint
    pointer that is not 16-byte aligned is refused."""
    import torch
    from frsppm import abi
    lib = abi.load()
    hp, R, ph = _inputs(23, 1000, 20_000)
    R[[3, 10, 500]] = [np.nan, np.inf, 10.0]
    cell = 0.04
    with abi.Renderer(GOLDEN_SCENES['cornell32'](), 16) as r:
        ok = np.ones(len(R), bool)
        ok[[3, 10, 500]] = False
        want, _ = r.radius_query(hp[ok], R[ok], ph, cell)
    hp_dev = torch.from_numpy(np.concatenate([hp, R[:, None]], 1)).cuda()
    ph_dev = torch.from_numpy(ph).cuda()
    out = torch.zeros(len(R), dtype=torch.int32, device='cuda')
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.fr_radius_count_noalloc(ctypes.c_void_p(hp_dev.data_ptr()), len(R), ctypes.c_void_p(ph_dev.data_ptr()),
                                     len(ph), ctypes.c_float(cell), ctypes.c_void_p(out.data_ptr()),
                                     ctypes.c_void_p(stream))
    assert rc == 0, lib.fr_last_error()
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert (got[~ok] == -1).all()
    np.testing.assert_array_equal(got[ok], want)
    flat = torch.zeros(4 * 8 + 1, dtype=torch.float32, device='cuda')
    rc = lib.fr_radius_count_noalloc(ctypes.c_void_p(flat.data_ptr() + 4), 8, ctypes.c_void_p(ph_dev.data_ptr()),
                                     len(ph), ctypes.c_float(cell), ctypes.c_void_p(out.data_ptr()),
                                     ctypes.c_void_p(stream))
    assert rc == 1 and b'aligned' in lib.fr_last_error()
