"""CPU-side checks: the C-ABI library loads and exports every symbol the
header declares; the golden fixtures match the scene generators."""
import importlib.util
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN_SCENES, REPO, load_golden


def test_header_and_binding_agree():
    from frsppm import abi
    hdr = open(os.path.join(REPO, 'include', 'friendsrender.h')).read()
    declared = set(re.findall(r'\b(fr_[a-z0-9_]+)\s*\(', hdr))
    assert declared == set(abi.EXPORTS)


def test_library_exports_every_symbol():
    from frsppm import abi
    lib = abi.load()
    for name in abi.EXPORTS:
        assert hasattr(lib, name), name


def test_last_error_without_gpu_call():
    from frsppm import abi
    lib = abi.load()
    assert isinstance(lib.fr_last_error(), bytes)


def _make_golden():
    spec = importlib.util.spec_from_file_location('make_golden', os.path.join(REPO, 'tests', 'golden', 'make_golden.py'))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.mark.parametrize('name', sorted(GOLDEN_SCENES))
def test_fixture_matches_scene_generator(name):
    gold = load_golden(name)
    assert str(gold['scene_sha']) == _make_golden().scene_sha(GOLDEN_SCENES[name]())


def test_scene_sizes():
    from frsppm import scenes
    assert len(scenes.cornell_box()['pos']) == 36
    s = scenes.small_mixed()
    assert {m['type'] for m in s['materials']} == {0, 1, 2, 3}
    assert all(t.dtype == np.uint8 and t.shape[2] == 4 for t in s['textures'])
