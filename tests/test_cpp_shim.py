"""The C++ mirror of the reference's render interface (include/friendsrender.hpp):
it compiles and links against libfrsppm.so and reads a scene back from OBJ
with fr::Scene::CreateScene (CPU), and on a GPU its RenderImage_FixStep
renders what the C-ABI calls render, from the arrays and from the OBJ
(tests/cpp)."""
import os
import subprocess

import pytest

from conftest import REPO

PKG = os.path.join(REPO, 'friendsrender-r-public_gb300')


def _build(tmp_path):
    exe = str(tmp_path / 'shim_check')
    cmd = ['g++', '-std=c++17', '-O1', '-I', os.path.join(REPO, 'include'), os.path.join(REPO, 'tests', 'cpp',
           'shim_check.cpp'), '-L', PKG, '-lfrsppm', '-Wl,-rpath,' + PKG, '-o', exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_compiles_links_and_loads_obj(tmp_path):
    """Builds the check and runs its host-only part: fr::Scene::CreateScene
    with a SceneMaterialManager reads back the OBJ/MTL it wrote."""
    if not os.path.exists(os.path.join(PKG, 'libfrsppm.so')):
        pytest.skip('library not built')
    exe = _build(tmp_path)
    r = subprocess.run([exe, str(tmp_path), 'ingest'], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith('ok'), r.stdout + r.stderr


@pytest.mark.gpu
def test_shim_renders_like_the_c_abi(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith('ok'), r.stdout + r.stderr
