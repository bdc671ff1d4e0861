"""The bound on a radius query's cell range (query_ball_ok in
csrc/fr_layout.h), checked on the CPU: balls that are not finite, or that
span more than 128 cells along an axis, are refused before any loop over
cells starts (fr_radius_query returns FR_ERR_INVALID, the kernels write the
count -1), and every accepted ball's cell range stays within that bound."""
import os
import subprocess

from conftest import REPO


def test_query_ball_bounds(tmp_path):
    exe = str(tmp_path / 'query_bounds_check')
    src = os.path.join(REPO, 'tests', 'cpp', 'query_bounds_check.cpp')
    inc = os.path.join(REPO, 'friendsrender-r-public_gb300', 'csrc')
    r = subprocess.run(['g++', '-std=c++17', '-O2', '-ffp-contract=off', '-I', inc, src, '-o', exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip().endswith('ok'), r.stdout + r.stderr
