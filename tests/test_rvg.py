"""RVG documents (spr_rvg_load / spr_rvg_parse, after RVG::load in rvg.cpp
and the fill conversion of addVg): element -> path, commands -> curves,
transforms, paints, and the reference's quirks (open contours closed only
at their element's end, Z adds no segment, rgb() drops a character).  The
document below is written for these tests; it is not one of the reference's
benchmark files."""
import numpy as np
import pytest

import oracle
import spr

L, Q, CU, R = spr.CURVE_LINEAR, spr.CURVE_QUADRATIC, spr.CURVE_CUBIC, spr.CURVE_RATIONAL

DOC = """viewport 0,0 200,150
window 0,0 200,150
scene dyn_identity
1 element nzfill dyn_concrete 0,0 0,0 0,0 M 10,10 L 90,10 L 90,60 L 10,60 L 10,10 Z dyn_identity dyn_paint 1 solid rgba(1,0,0,1)
// a comment line
1 element ofill dyn_concrete 0,0 0,0 0,0 M 20,20 Q 60,0 100,20 C 120,40 80,80 20,70 dyn_affine[[1,0,5],[0,1,7]] dyn_paint 0.5 solid rgb(0,0.5,0.25)
1 element nzfill dyn_concrete 0,0 0,0 0,0 M 150,75 A 20,0,0 150,115 fL 10,140 M 120,120 A 20,0,0.5 160,120 dyn_identity dyn_paint 1 solid rgba(0,0,1,0.6)
1 element xfill dyn_concrete 0,0 0,0 0,0 M 0,0 L 1,1 dyn_identity dyn_paint 1 solid rgba(1,1,1,1)
1 element nzfill dyn_concrete 0,0 0,0 0,0 M 30,100 L 70,100 L 50,140 dyn_identity dyn_paint 1 linear 0,0 1,0 0 0 0 0 1 1 1 1 1 1 pad 1 0 0 0 1 0
1 element nzfill dyn_concrete 0,0 0,0 0,0 M 5,5 L 6,5 L 6,6 Z dyn_identity dyn_paint 1 solid rgba(1,1,1,0)
"""


def curves_of(sc):
    out = []
    for c in range(len(sc.curve_type)):
        p0, n = sc.curve_vertex_pos[c], sc.curve_type[c] & 7
        pts = [tuple(map(float, sc.vertex[p0 + k])) for k in range(n)]
        out.append((int(sc.curve_path_id[c]), int(sc.curve_type[c]), pts, float(sc.curve_arc_w[c])))
    return out


def test_parse_paths_curves_and_paints():
    sc, info = spr.Scene.parse_rvg(DOC)
    assert info["viewport"] == [0, 0, 200, 150] and info["window"] == [0, 0, 200, 150]
    assert (info["width"], info["height"], info["n_elements"], info["n_gradient_paths"]) == (200, 150, 6, 1)
    assert sc.n_paths == 5
    assert sc.path_fill_rule.tolist() == [0, 1, 0, 0, 0]
    # rgba(1,0,0,1); rgb(0,0.5,0.25) read as (0, 0.5, 0.2) at opacity 0.5; alpha 0.6;
    # a linear paint (gradient index path + 1); alpha 0 -> 0
    assert sc.path_fill_rgba.tolist() == [0xFF0000FF, 0x7F337F00, 0x99FF0000, 4, 0]
    q = 0.7071067690849304  # float(0.70710678...)
    exp = [
        (0, L, [(10, 10), (90, 10)], -1), (0, L, [(90, 10), (90, 60)], -1), (0, L, [(90, 60), (10, 60)], -1),
        (0, L, [(10, 60), (10, 10)], -1),
        # translated by (5, 7), closed by a line back to the contour's start
        (1, Q, [(25, 27), (65, 7), (105, 27)], -1), (1, CU, [(105, 27), (125, 47), (85, 87), (25, 77)], -1),
        (1, L, [(25, 77), (25, 27)], -1),
        # half circle as two quarter arcs; fL moves without a segment; the last
        # contour (an arc of weight 0.5, middle point (20,0)/0.5) is closed
        (2, R, [(150, 75), (170, 75), (170, 95)], q), (2, R, [(170, 95), (170, 115), (150, 115)], q),
        (2, R, [(120, 120), (40, 0), (160, 120)], 0.5), (2, L, [(160, 120), (120, 120)], -1),
        # the skipped element's path is taken by the next element
        (3, L, [(30, 100), (70, 100)], -1), (3, L, [(70, 100), (50, 140)], -1), (3, L, [(50, 140), (30, 100)], -1),
        # Z adds no segment
        (4, L, [(5, 5), (6, 5)], -1), (4, L, [(6, 5), (6, 6)], -1),
    ]
    got = curves_of(sc)
    assert len(got) == len(exp)
    for g, e in zip(got, exp):
        assert g[0] == e[0] and g[1] == e[1], (g, e)
        assert np.allclose(g[2], e[2]) and g[3] == pytest.approx(e[3]), (g, e)
    assert np.array_equal(sc.vertex_path_id, np.repeat([c[0] for c in got], [c[1] & 7 for c in got]))
    assert spr.lib().spr_validate_scene(sc.view()) == spr.OK


def test_alpha_options_and_errors(tmp_path):
    sc, _ = spr.Scene.parse_rvg(DOC, a128=True)
    # 7-bit alpha: 255 -> 127 -> 255, 127 -> 63 -> 126, 153 -> 76 -> 152
    assert [c >> 24 for c in sc.path_fill_rgba.tolist()] == [255, 126, 152, 0, 0]
    f = tmp_path / "doc.rvg"
    f.write_text(DOC)
    a, ia = spr.Scene.load_rvg(f)
    b, ib = spr.Scene.parse_rvg(DOC)
    assert ia == ib and all(np.array_equal(getattr(a, k), getattr(b, k)) for k in spr.Scene.FIELDS
                            if getattr(a, k) is not None)
    head = "viewport 0,0 10,10\nwindow 0,0 10,10\nscene dyn_identity\n"
    with pytest.raises(spr.SprError) as e:  # relative commands
        spr.Scene.parse_rvg(head + "1 element nzfill dyn_concrete 0,0 0,0 0,0 M 1,1 l 2,2 dyn_identity "
                                   "dyn_paint 1 solid rgba(1,1,1,1)\n")
    assert e.value.status == spr.ERR_UNSUPPORTED
    for bad in ["1 element nzfill dyn_concrete 0,0 0,0 0,0 M 1,1 L 2,2 dyn_oops dyn_paint 1 solid rgba(1,1,1,1)\n",
                "2 element nzfill dyn_concrete 0,0 0,0 0,0 M 1,1 L 2,2 dyn_identity dyn_paint 1 solid rgba(1,1,1,1)\n",
                "1 element nzfill dyn_concrete 0,0 0,0 0,0 M 1,1 L 2,2 dyn_identity dyn_paint 1 solid hsl(1,1,1)\n",
                "1 element nzfill dyn_concrete 0,0 0,0 0,0 M 1,1 L 2,2"]:
        with pytest.raises(spr.SprError) as e:
            spr.Scene.parse_rvg(head + bad)
        assert e.value.status == spr.ERR_INVALID_SCENE
    with pytest.raises(spr.SprError) as e:
        spr.Scene.load_rvg(tmp_path / "missing.rvg")
    assert e.value.status == spr.ERR_INVALID_ARG


def test_oracle_renders_a_loaded_document():
    sc, info = spr.Scene.parse_rvg(DOC)
    img = oracle.run(sc, info["width"], info["height"], samples=8, srgb=False)["IMAGE"]
    img = img.reshape(info["height"], info["width"], 4)
    assert img[15, 15].tolist() == [255, 0, 0, 255]     # inside the red square only
    assert img[120, 50].tolist() == [255, 255, 255, 255]  # the gradient triangle is not drawn
    assert img[2, 190].tolist() == [255, 255, 255, 255]   # background


@pytest.mark.gpu
def test_gpu_parity_on_a_loaded_document():
    sc, info = spr.Scene.parse_rvg(DOC)
    W, H = info["width"], info["height"]
    for samples in (8, 32):
        ref = oracle.run(sc, W, H, samples=samples)["IMAGE"]
        with spr.VGRasterizer(W, H, samples=samples) as r:
            r.add_vg(sc)
            r.rasterize()
            assert np.array_equal(r.read_image().reshape(-1), ref)
