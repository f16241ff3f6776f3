"""The reference's scene files (.vgb binary, .vgt text; VGContainer::save /
load) through spr_vg_load / spr_vg_save, flattened as addVg does."""
import struct

import numpy as np
import pytest

import oracle
import spr
from test_rvg import DOC

FIELDS = ("vertex", "vertex_path_id", "curve_vertex_pos", "curve_type", "curve_path_id", "curve_arc_w",
          "path_fill_rule", "path_fill_rgba")


def same(a, b, vertex_rtol=0.0):
    for f in FIELDS:
        x, y = getattr(a, f), getattr(b, f)
        if f == "vertex" and vertex_rtol:
            assert np.allclose(x, y, rtol=vertex_rtol, atol=0), f
        else:
            assert np.array_equal(x, y), f


@pytest.mark.parametrize("suffix", ["vgb", "vgt"])
def test_round_trip(tmp_path, suffix):
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=5, width=256, height=200, n_paths=40, n_large=4,
                            with_rational=True)
    f = tmp_path / f"scene.{suffix}"
    sc.save_vg(f, 256, 200)
    back, info = spr.Scene.load_vg(f)
    assert (info["width"], info["height"], info["n_contours"]) == (256, 200, sc.n_paths)
    same(back, sc, vertex_rtol=1e-6 if suffix == "vgt" else 0.0)  # %e keeps 7 significant digits
    assert back.gradients is None


def test_rvg_document_with_gradients_round_trips(tmp_path):
    sc, info = spr.Scene.parse_rvg(DOC)
    f = tmp_path / "doc.vgb"
    sc.save_vg(f, info["width"], info["height"])
    back, _ = spr.Scene.load_vg(f)
    same(back, sc)
    assert all(np.array_equal(x, y) for x, y in zip(back.gradients, sc.gradients))
    a = oracle.run(sc, info["width"], info["height"], samples=8)["IMAGE"]
    b = oracle.run(back, info["width"], info["height"], samples=8)["IMAGE"]
    assert np.array_equal(a, b)


def vgb(paths, contours, curves, vertices, ramp=(), table=(), xywh=(0, 0, 64, 48)):
    """A .vgb file from records: paths (contour index, contour count, fill
    type, fill rule, rgba, fill index), contours (curve index, count), curves
    (vertex index, type, weight float), vertices (x, y)."""
    b = struct.pack("<4i6I", *xywh, len(paths), len(contours), len(curves), len(vertices), len(ramp), len(table))
    b += b"".join(struct.pack("<I", p[0]) for p in paths) + b"".join(struct.pack("<I", p[1]) for p in paths)
    b += bytes(p[2] for p in paths) + bytes(p[3] for p in paths)
    b += b"".join(struct.pack("<I", p[4]) for p in paths) + b"".join(struct.pack("<I", p[5]) for p in paths)
    b += b"".join(struct.pack("<I", c[0]) for c in contours) + b"".join(struct.pack("<I", c[1]) for c in contours)
    b += b"".join(struct.pack("<I", c[0]) for c in curves) + bytes(c[1] for c in curves)
    b += b"".join(struct.pack("<f", c[2]) for c in curves)
    b += b"".join(struct.pack("<2f", *v) for v in vertices)
    b += b"".join(struct.pack("<I", v) for v in ramp) + b"".join(struct.pack("<I", v) for v in table)
    return b


def test_flattening_follows_add_vg(tmp_path):
    """Two contours in one path, contours listed out of path order, a colour
    with alpha 0, a gradient fill, an even-odd rule and a rational curve."""
    Lc, Qc, Rc = spr.CURVE_LINEAR, spr.CURVE_QUADRATIC, spr.CURVE_RATIONAL
    verts = [(1, 1), (9, 1), (9, 1), (9, 9), (9, 9), (1, 1),          # path 0 contour A: curves 0-2
             (20, 20), (30, 20), (25, 30), (25, 30), (20, 20),         # path 1: curves 3 (quad), 4
             (40, 5), (50, 5), (50, 5), (45, 15), (40, 5),             # path 0 contour B: 5 (rational), 6
             (2, 30), (12, 30), (12, 30), (2, 40), (2, 40), (2, 30)]   # path 2: 7-9
    curves = [(0, Lc, 0), (2, Lc, 0), (4, Lc, 0), (6, Qc, 0), (9, Lc, 0), (11, Rc, 0.5), (14, Lc, 0),
              (16, Lc, 0), (18, Lc, 0), (20, Lc, 0)]
    contours = [(0, 3), (5, 2), (3, 2), (7, 3)]  # path 0 = contours 0, 1 (curves 0-2, 5-6)
    paths = [(0, 2, 1, 0, 0xFF0000FF, 0xFFFFFFFF), (2, 1, 1, 1, 0x00ABCDEF, 0xFFFFFFFF),
             (3, 1, 4, 0, 0x00FF00FF, 0)]
    f = tmp_path / "h.vgb"
    f.write_bytes(vgb(paths, contours, curves, verts, ramp=[0] * 1024, table=[0] * 36))
    # addVg numbers vertex paths curve by curve, whatever the vertices' order
    sc, _ = spr.Scene.load_vg(f)
    assert sc.curve_path_id.tolist() == [0, 0, 0, 0, 0, 1, 1, 2, 2, 2]
    assert sc.curve_vertex_pos.tolist() == [0, 2, 4, 11, 14, 6, 9, 16, 18, 20]
    assert sc.vertex_path_id.tolist() == [0] * 11 + [1] * 5 + [2] * 6
    # curves whose vertex counts do not add up to the vertices: refused
    f.write_bytes(vgb(paths, contours, curves[:-1], verts, ramp=[0] * 1024, table=[0] * 36))
    with pytest.raises(spr.SprError) as e:
        spr.Scene.load_vg(f)
    assert e.value.status == spr.ERR_INVALID_SCENE
    # in array order: path 0 = contours 0 and 1 over curves 0-2 and 3-4
    verts2 = verts[:6] + verts[11:16] + verts[6:11] + verts[16:]
    curves2 = [(0, Lc, 0), (2, Lc, 0), (4, Lc, 0), (6, Rc, 0.5), (9, Lc, 0), (11, Qc, 0), (14, Lc, 0),
               (16, Lc, 0), (18, Lc, 0), (20, Lc, 0)]
    contours2 = [(0, 3), (3, 2), (5, 2), (7, 3)]
    f.write_bytes(vgb(paths, contours2, curves2, verts2, ramp=[0] * 1024, table=[0] * 36))
    sc, info = spr.Scene.load_vg(f)
    assert (info["width"], info["height"], info["n_contours"]) == (64, 48, 4)
    assert sc.path_fill_rgba.tolist() == [0xFF0000FF, 0, 3]   # alpha 0 -> 0; gradient -> path + 1
    assert sc.path_fill_rule.tolist() == [0, 1, 0]
    assert sc.curve_path_id.tolist() == [0, 0, 0, 0, 0, 1, 1, 2, 2, 2]
    assert sc.curve_type.tolist() == [c[1] for c in curves2]
    assert sc.curve_arc_w[3] == 0.5 and sc.curve_arc_w[0] == -1
    assert np.array_equal(sc.vertex, np.array(verts2, np.float32))
    assert sc.gradients is not None and len(sc.gradients[1]) == 1024


def test_errors(tmp_path):
    sc = spr.Scene.generate(spr.SCENE_RANDOM, seed=2, width=64, height=64, n_paths=4)
    f = tmp_path / "s.vgb"
    sc.save_vg(f, 64, 64)
    data = f.read_bytes()
    f.write_bytes(data[:-5])
    with pytest.raises(spr.SprError) as e:
        spr.Scene.load_vg(f)
    assert e.value.status == spr.ERR_INVALID_SCENE
    with pytest.raises(spr.SprError) as e:
        spr.Scene.load_vg(tmp_path / "s.svg")
    assert e.value.status == spr.ERR_INVALID_ARG
    aff = spr.Scene.generate(spr.SCENE_MIXED, seed=3, width=64, height=64, n_paths=4, with_affine=True)
    with pytest.raises(spr.SprError) as e:
        aff.save_vg(tmp_path / "a.vgb", 64, 64)
    assert e.value.status == spr.ERR_UNSUPPORTED
