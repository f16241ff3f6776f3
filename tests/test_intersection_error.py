"""The FP64 check of the crossing points (oracle.intersection_error), on the
CPU: it follows the same walk as the entries (no mismatches), the FP32
crossings of the small plain-path workload lie within a small fraction of a
pixel of the exact FP64 crossings, and a planted error in an entry is seen."""
import numpy as np

import oracle
import spr


def small_scene():
    return spr.Scene.generate(spr.SCENE_RANDOM, seed=20261203, width=512, height=512, n_paths=64, seg_min=8,
                              seg_max=32)


def test_small_workload_crossings_are_accurate():
    sc = small_scene()
    ref = oracle.run(sc, 512, 512, samples=8)
    e = oracle.intersection_error(sc, ref["TVERTEX"], ref["INTERSECTION"], 512, 512)
    # every entry is a piece start or a crossing of the walk
    assert e["n_mismatched"] == 0
    assert 0.9 * ref.counts["curve_fragment"] < e["n_crossings"] < ref.counts["curve_fragment"]
    assert e["n_over_1px"] == 0 and e["max_err_px"] < 0.05 and e["mean_err_px"] < 1e-3
    assert e["max_resid_px"] < 0.01


def test_rational_and_transformed_curves():
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=3, width=384, height=320, n_paths=200, n_large=8,
                            with_rational=True, with_affine=True)
    tf = np.eye(4, dtype=np.float32)
    tf[0, :2] = [1.1, 0.3]
    tf[1, :2] = [-0.2, 0.9]
    tf[3, :2] = [2e-4, -1e-4]
    ref = oracle.run(sc, 384, 320, samples=8, transform=tf)
    e = oracle.intersection_error(sc, ref["TVERTEX"], ref["INTERSECTION"], 384, 320)
    assert e["n_mismatched"] == 0 and e["n_crossings"] > 10_000
    assert e["max_err_px"] < 0.05 and e["n_unbracketed"] < 1e-3 * e["n_crossings"]


def test_planted_errors_are_reported():
    sc = small_scene()
    ref = oracle.run(sc, 512, 512, samples=8)
    tv, en = ref["TVERTEX"].copy(), ref["INTERSECTION"].reshape(-1, 2).copy()
    base = oracle.intersection_error(sc, tv, en, 512, 512)
    # an entry whose t is not the walk's: counted, not measured
    k = len(en) // 2
    en[k, 1] = np.int32(np.float32(0.5).view(np.int32) | (en[k, 1] & 3))
    e = oracle.intersection_error(sc, tv, en, 512, 512)
    assert e["n_mismatched"] >= 1
    # a vertex moved after the entries were solved: its crossings are off
    tv2 = tv.copy()
    p = int(sc.curve_vertex_pos[5])
    tv2[p + 1] += np.float32(3.0)
    e2 = oracle.intersection_error(sc, tv2, ref["INTERSECTION"], 512, 512)
    assert e2["n_mismatched"] > 0 or e2["max_err_px"] > base["max_err_px"]


def test_exact_line_crossings():
    """A single straight edge: the exact crossings are known in closed form."""
    v = np.array([[0.3, 0.1], [40.7, 30.9], [40.7, 30.9], [0.3, 30.9], [0.3, 30.9], [0.3, 0.1]], np.float32)
    sc = spr.Scene(v, np.zeros(6, np.uint32), np.array([0, 2, 4], np.uint32),
                   np.full(3, spr.CURVE_LINEAR, np.uint8), np.zeros(3, np.uint32), np.full(3, -1, np.float32),
                   np.zeros(1, np.uint8), np.array([0xFF0000FF], np.uint32))
    ref = oracle.run(sc, 48, 40, samples=8)
    e = oracle.intersection_error(sc, ref["TVERTEX"], ref["INTERSECTION"], 48, 40)
    assert e["n_mismatched"] == 0 and e["n_crossings"] > 30 and e["max_err_px"] < 1e-3
