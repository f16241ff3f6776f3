"""The C ABI library (no GPU needed): exports, status strings, the synthetic
scene generator and host-side scene validation."""
import ctypes as C
import pathlib
import re

import numpy as np
import pytest

import spr

ROOT = pathlib.Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "spr.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(spr_\w+)\s*\(", text)))


def test_library_exports_every_declared_function():
    L = spr.lib()
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_oracle_is_separate_library():
    import oracle

    assert oracle.LIB_PATH.exists()
    assert not hasattr(spr.lib(), "orc_run")  # the product never links the oracle


def test_status_strings():
    for st in range(0, 9):
        assert spr.lib().spr_status_string(st)
    assert b"unknown" in spr.lib().spr_status_string(99)


@pytest.mark.parametrize("kind", [spr.SCENE_RANDOM, spr.SCENE_MIXED, spr.SCENE_CUBICS, spr.SCENE_LOCAL])
def test_generator_deterministic_and_valid(kind):
    a = spr.Scene.generate(kind, seed=5, width=300, height=200, n_paths=30, n_large=4, seg_min=8,
                           seg_max=20, with_rational=True, with_affine=True)
    b = spr.Scene.generate(kind, seed=5, width=300, height=200, n_paths=30, n_large=4, seg_min=8,
                           seg_max=20, with_rational=True, with_affine=True)
    c = spr.Scene.generate(kind, seed=6, width=300, height=200, n_paths=30, n_large=4, seg_min=8,
                           seg_max=20, with_rational=True, with_affine=True)
    for f in spr.Scene.FIELDS:
        x, y = getattr(a, f), getattr(b, f)
        assert (x is None and y is None) or np.array_equal(x, y), f
    assert not np.array_equal(a.vertex, c.vertex)
    assert a.validate() == spr.OK
    # curves are grouped by path and each path is a closed contour
    assert np.all(np.diff(a.curve_path_id.astype(np.int64)) >= 0)
    n = a.curve_type & 7
    first = a.vertex[a.curve_vertex_pos]
    last = a.vertex[a.curve_vertex_pos + n - 1]
    for p in range(a.n_paths):
        idx = np.nonzero(a.curve_path_id == p)[0]
        assert np.array_equal(last[idx[:-1]], first[idx[1:]])
        assert np.array_equal(last[idx[-1]], first[idx[0]])
    assert set(np.unique(a.curve_type)) <= {2, 3, 4, 0x13}
    alpha = a.path_fill_rgba >> 24
    assert np.all((alpha >= 127) & (alpha <= 255))


def test_random_scene_segment_counts():
    s = spr.Scene.generate(spr.SCENE_RANDOM, seed=9, width=512, height=512, n_paths=64, seg_min=8, seg_max=32)
    per_path = np.bincount(s.curve_path_id, minlength=64)
    assert per_path.min() >= 8 and per_path.max() <= 32
    frac = np.bincount(s.curve_type, minlength=5)[2:5] / s.n_curves
    assert abs(frac[0] - 0.4) < 0.06 and abs(frac[1] - 0.3) < 0.06 and abs(frac[2] - 0.3) < 0.06


def _bad(scene, **changes):
    s = scene.copy()
    for k, v in changes.items():
        setattr(s, k, v)
    return s.validate()


def test_validation_rejects_malformed_scenes():
    s = spr.Scene.generate(spr.SCENE_RANDOM, seed=3, width=64, height=64, n_paths=4, seg_min=3, seg_max=5)
    assert s.validate() == spr.OK
    t = s.curve_type.copy()
    t[1] = 7
    assert _bad(s, curve_type=t) == spr.ERR_INVALID_SCENE
    vp = s.curve_vertex_pos.copy()
    vp[-1] = s.n_vertices
    assert _bad(s, curve_vertex_pos=vp) == spr.ERR_INVALID_SCENE
    pid = s.curve_path_id.copy()
    pid[0], pid[-1] = pid[-1], pid[0]
    assert _bad(s, curve_path_id=pid) == spr.ERR_INVALID_SCENE
    vpid = s.vertex_path_id.copy()
    vpid[0] = 99
    assert _bad(s, vertex_path_id=vpid) == spr.ERR_INVALID_SCENE
    v = s.view()
    v.vertex = None
    assert spr.lib().spr_validate_scene(C.byref(v)) == spr.ERR_INVALID_ARG
    assert spr.lib().spr_validate_scene(None) == spr.ERR_INVALID_ARG


def test_create_without_gpu_fails_cleanly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    cfg = spr.Config(64, 64, 8, 1, 1, 0)
    h = C.c_void_p()
    st = spr.lib().spr_create(C.byref(cfg), C.byref(h))
    assert st in (spr.ERR_CUDA, spr.ERR_INVALID_ARG) and not h.value


def test_create_rejects_bad_config_before_touching_the_device():
    for cfg in (spr.Config(0, 64, 8, 1, 1, 0), spr.Config(64, 5000, 8, 1, 1, 0), spr.Config(64, 64, 12, 1, 1, 0)):
        h = C.c_void_p()
        assert spr.lib().spr_create(C.byref(cfg), C.byref(h)) == spr.ERR_INVALID_ARG


def test_local_scene_paths_stay_in_their_boxes():
    s = spr.Scene.generate(spr.SCENE_LOCAL, seed=12, width=1024, height=768, n_paths=200, seg_min=8, seg_max=32)
    assert s.validate() == spr.OK and s.n_paths == 200
    for p in range(s.n_paths):
        v = s.vertex[s.vertex_path_id == p]
        ext = v.max(axis=0) - v.min(axis=0)
        assert ext.max() <= 768 / 4 + 1e-3


def test_batch_create_without_gpu_fails_cleanly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert spr.lib().spr_batch_create(0, 1, 1, C.byref(h)) == spr.ERR_CUDA and not h.value
    assert spr.lib().spr_batch_create(0, 1, 1, None) == spr.ERR_INVALID_ARG
    assert spr.lib().spr_batch_render(None, None) == spr.ERR_INVALID_ARG
