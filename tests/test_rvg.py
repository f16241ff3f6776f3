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
1 element nzfill dyn_concrete 0,0 0,0 0,0 M 30,100 L 70,100 L 50,140 dyn_identity dyn_paint 1 linear 30,0 70,0 0 1 0 0 1 1 0 0 1 1 pad 1 0 0 0 1 0
1 element nzfill dyn_concrete 0,0 0,0 0,0 M 5,5 L 6,5 L 6,6 Z dyn_identity dyn_paint 1 solid rgba(1,1,1,0)
1 element nzfill dyn_concrete 0,0 0,0 0,0 M 110,80 L 190,80 L 190,140 L 110,140 L 110,80 dyn_identity dyn_paint 0.8 radial 150,110 150,110 30 0 1 1 0 1 1 0 0 1 1 pad 1 0 0 0 1 0
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
    assert (info["width"], info["height"], info["n_elements"], info["n_gradient_paths"]) == (200, 150, 7, 2)
    assert sc.n_paths == 6
    assert sc.path_fill_rule.tolist() == [0, 1, 0, 0, 0, 0]
    # rgba(1,0,0,1); rgb(0,0.5,0.25) read as (0, 0.5, 0.2) at opacity 0.5; alpha 0.6;
    # a linear paint (gradient index path + 1); alpha 0 -> 0; a radial paint
    assert sc.path_fill_rgba.tolist() == [0xFF0000FF, 0x7F337F00, 0x99FF0000, 4, 0, 6]
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
        (5, L, [(110, 80), (190, 80)], -1), (5, L, [(190, 80), (190, 140)], -1),
        (5, L, [(190, 140), (110, 140)], -1), (5, L, [(110, 140), (110, 80)], -1),
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
    assert [c >> 24 for c in sc.path_fill_rgba.tolist()] == [255, 126, 152, 0, 0, 0]
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


def test_gradient_table_and_ramps():
    """One 12-word table entry per painted path (solid paths: empty slots),
    ramps packed by decreasing length inside 1024-texel rows, the linear
    paint's map taking x = 30..70 to gradient x = -1..1, the radial one's
    scaled by 1/r with the focal point at the centre."""
    sc, _ = spr.Scene.parse_rvg(DOC, srgb_ramps=False)
    table, ramp = sc.gradients
    assert len(table) == 12 * 6 and len(ramp) % 1024 == 0
    t = table.view(np.float32).reshape(6, 12)
    ti = table.view(np.int32).reshape(6, 12)
    for e in (0, 1, 2, 4):  # solid slots
        assert t[e, 7] == np.float32(-1 / 1024)
    lin, rad = t[3], t[5]
    assert np.allclose(lin[:6], [2 / 40, 0, -1 - 60 / 40, 0, 0, 0]) and np.allclose(lin[8:11], [-1, 0, 0])
    assert np.allclose(rad[:6], [1 / 30, 0, -150 / 30, 0, 1 / 30, -110 / 30]) and np.allclose(rad[8:11], [0, 0, 1])
    n_lin, n_rad = round(lin[7] * 1024) + 1, round(rad[7] * 1024) + 1
    assert n_lin == n_rad == 32  # 16 / (smallest stop gap 1), rounded up past a power of two
    p_lin, p_rad = ti[3, 6], ti[5, 6]
    assert {p_lin, p_rad} == {0, 32}
    r_lin = ramp[p_lin:p_lin + 32]
    assert r_lin[0] == 0xFF0000FF and (r_lin[-1] & 0xFFFFFF) in (0xFE0000, 0xFF0000)  # red -> blue
    red = r_lin & 0xFF
    assert np.all(np.diff(red.astype(int)) <= 0)
    r_rad = ramp[p_rad:p_rad + 32]
    assert (r_rad[0] >> 24) == int(0.8 * 255) and (r_rad[0] & 0xFFFFFF) == 0x00FFFF  # yellow at 0.8 opacity


def test_oracle_renders_a_loaded_document():
    sc, info = spr.Scene.parse_rvg(DOC, srgb_ramps=False)
    img = oracle.run(sc, info["width"], info["height"], samples=8, srgb=False)["IMAGE"]
    img = img.reshape(info["height"], info["width"], 4)
    assert img[15, 15].tolist() == [255, 0, 0, 255]     # inside the red square only
    assert img[2, 190].tolist() == [255, 255, 255, 255]   # background
    row = img[104, 34:67]                                # across the linear gradient: red to blue
    assert np.all(np.diff(row[:, 0].astype(int)) <= 0) and np.all(np.diff(row[:, 2].astype(int)) >= 0)
    assert row[0, 0] > 200 and row[-1, 2] > 200
    # radial: yellow at the centre, bluer outwards, alpha 0.8 over white
    c, edge = img[110, 150], img[110, 176]
    assert c[0] > 200 and c[1] > 200 and c[2] < 80 and edge[2] > c[2]


@pytest.mark.gpu
@pytest.mark.parametrize("srgb", [True, False])
@pytest.mark.parametrize("ms", [True, False])
def test_gpu_parity_on_a_loaded_document(srgb, ms):
    """The loaded document, gradient paints included, bit-exact against the
    oracle; a reverse transform (scaling the gradient coordinates) too."""
    sc, info = spr.Scene.parse_rvg(DOC, srgb_ramps=srgb)
    W, H = info["width"], info["height"]
    rev = np.array([1.1, 0, 0, 0, 0.9, 0, -3, 2, 1, 0, 0, 0, 1], np.float32)
    for samples in (8, 32):
        for rv in (None, rev):
            ref = oracle.run(sc, W, H, samples=samples, ms_output=ms, srgb=srgb, rev=rv)["IMAGE"]
            with spr.VGRasterizer(W, H, samples=samples, ms_output=ms, srgb=srgb) as r:
                r.add_vg(sc)
                if rv is not None:
                    r.set_rev_transform(rv)
                r.rasterize()
                assert np.array_equal(r.read_image().reshape(-1), ref), (samples, rv is not None)
