"""SVG documents (spr_svg_load / spr_svg_parse, after SVG::load in
svg_load.cpp and the fill conversion of addVg): elements, inherited
presentation attributes, transforms, path data with the reference's reading
(moves, closes, reflections, arcs as cubics), the viewBox flip, gradient
fills, strokes, and the documents the reference cannot read.  The documents
below are written for these tests."""
import math

import numpy as np
import pytest

import oracle
import spr

L, Q, CU, R = spr.CURVE_LINEAR, spr.CURVE_QUADRATIC, spr.CURVE_CUBIC, spr.CURVE_RATIONAL

DOC = """<?xml version="1.0" encoding="UTF-8"?>
<!DOCTYPE svg PUBLIC "-//W3C//DTD SVG 1.1//EN" "http://www.w3.org/Graphics/SVG/1.1/DTD/svg11.dtd" [
  <!ENTITY nothing "">
]>
<svg width="200" height="100" viewBox="0 0 200 100" xmlns="http://www.w3.org/2000/svg">
 <!-- a comment <path d="M0 0 L 1 1"/> -->
 <title>shapes &amp; paints</title>
 <defs>
  <linearGradient id="g" x1="10" y1="0" x2="90" y2="0" gradientUnits="userSpaceOnUse">
   <stop offset="0" stop-color="#ff0000"/>
   <stop offset="1" style="stop-color:#0000ff;stop-opacity:0.5"/>
  </linearGradient>
  <radialGradient id="r" cx="40" cy="40" r="30"><stop offset="0" stop-color="#ffff00"/>
   <stop offset="1" stop-color="#00f"/></radialGradient>
 </defs>
 <g fill="#00ff00" transform="translate(10, 5)">
  <path d="M0,0 L50,0 L50,40 z" fill-opacity="0.5"/>
  <path d="M60 0 h30 v30 h-30 z" fill="url(#g)" fill-rule="evenodd"/>
 </g>
 <polygon points="100,10 150,10 125,60" fill="rgb(10,20,30)" stroke="#123" stroke-width="4"/>
 <path d="M160,50 a20,20 0 1,0 30,0 z" fill="#abc"/>
 <path d="M10,60 L70,60 L70,95 L10,95 Z" fill="url(#r)"/>
 <foo><path d="M0 0 L 5 5 L 0 5 z"/></foo>
</svg>"""


def curves_of(sc):
    out = []
    for c in range(sc.n_curves):
        p0, n = sc.curve_vertex_pos[c], sc.curve_type[c] & 7
        out.append((int(sc.curve_path_id[c]), int(sc.curve_type[c]), sc.vertex[p0:p0 + n].tolist()))
    return out


def one(d, extra="", w=100, h=100):
    sc, _ = spr.Scene.parse_svg(f'<svg viewBox="0 0 {w} {h}"><path d="{d}" {extra}/></svg>')
    return sc


def unflip(pts, h=100):
    return [[x, h - y] for x, y in pts]


def test_document_paths_paints_and_flip():
    sc, info = spr.Scene.parse_svg(DOC)
    assert info == {"view_box": [0.0, 0.0, 200.0, 100.0], "width": 200, "height": 100, "n_paths": 5,
                    "n_gradient_paths": 2, "n_stroked_paths": 1}
    # green at fill-opacity 0.5 (255 * 0.5 -> 127); a gradient (path + 1); the
    # polygon filled with its stroke colour #123 (addVg); #abc; a radial gradient
    assert sc.path_fill_rgba.tolist() == [0x7F00FF00, 2, 0xFF332211, 0xFFCCBBAA, 5]
    assert sc.path_fill_rule.tolist() == [0, 1, 0, 0, 0]
    c = curves_of(sc)
    # translate(10, 5), then y flipped about the viewBox height
    assert [x[2] for x in c if x[0] == 0] == [unflip(p) for p in ([[10, 5], [60, 5]], [[60, 5], [60, 45]],
                                                                    [[60, 45], [10, 5]])]
    assert [x[2] for x in c if x[0] == 1] == [unflip(p) for p in (
        [[70, 5], [100, 5]], [[100, 5], [100, 35]], [[100, 35], [70, 35]], [[70, 35], [70, 5]])]
    assert [x[2] for x in c if x[0] == 2] == [unflip(p) for p in (
        [[100, 10], [150, 10]], [[150, 10], [125, 60]], [[125, 60], [100, 10]])]
    arc = [x for x in c if x[0] == 3]
    assert [x[1] for x in arc] == [CU, CU, CU, L]  # a large arc of three quarter turns or less, then Z
    assert np.allclose(arc[0][2][0], unflip([[160, 50]])[0]) and np.allclose(arc[2][2][3], unflip([[190, 50]])[0],
                                                                           atol=1e-4)
    table, ramp = sc.gradients
    t = table.view(np.float32).reshape(-1, 12)
    assert t.shape[0] == 5 and t[0, 7] == np.float32(-1 / 1024) and t[1, 7] > 0 and t[4, 7] > 0
    assert spr.lib().spr_validate_scene(sc.view()) == spr.OK


def test_path_data_reading():
    # relative commands; coordinates after the first pair of an M stay moves;
    # numbers split by '-' and written with exponents
    sc = one("m10 10 5 5 l10 0 l0-10 L1e1,10 z")
    assert curves_of(sc) == [(0, L, unflip([[15, 15], [25, 15]])), (0, L, unflip([[25, 15], [25, 5]])),
                             (0, L, unflip([[25, 5], [10, 10]])), (0, L, unflip([[10, 10], [15, 15]]))]
    # Z keeps the current point (and the contour: no line closes it again at
    # the next M); a new M after curves starts a contour
    sc = one("M0 0 L10 0 L10 10 Z l5 0 M50 50 L60 50 Z")
    assert [x[2] for x in curves_of(sc)] == [unflip(p) for p in (
        [[0, 0], [10, 0]], [[10, 0], [10, 10]], [[10, 10], [0, 0]], [[10, 10], [15, 10]],
        [[50, 50], [60, 50]], [[60, 50], [50, 50]])]
    # S reflects the last control point; Q and H / V
    sc = one("M0 0 C10 0 20 10 20 20 S30 40 40 40 Q50 50 60 40 H70 V50 h-5 v-5")
    c = curves_of(sc)
    assert [x[1] for x in c] == [CU, CU, Q, L, L, L, L]
    assert c[1][2] == unflip([[20, 20], [20, 30], [30, 40], [40, 40]])
    assert c[3][2] == unflip([[60, 40], [70, 40]]) and c[4][2] == unflip([[70, 40], [70, 50]])
    assert c[6][2] == unflip([[65, 50], [65, 45]])
    # a T after Z is passed over like any unknown character in command position
    sc = one("M0 0 L10 0 L0 10 Z T 5 5")
    assert sc.n_curves == 3


@pytest.mark.parametrize("flags", ["0 0", "1 0", "0 1", "1 1"])
def test_arcs_are_cubics_on_the_ellipse(flags):
    """Each arc's cubics start and end on the ellipse (rotated 30 degrees)
    and stay within 0.1 % of it; the arc ends at its end point."""
    rx, ry, rot = 30.0, 15.0, 30.0
    sc = one(f"M20 50 A{rx} {ry} {rot} {flags} 60 60")
    c = curves_of(sc)
    assert all(x[1] == CU for x in c) and 1 <= len(c) <= 4
    pts = [unflip([p])[0] for p in (c[0][2][0], c[-1][2][3])]
    assert np.allclose(pts[0], [20, 50], atol=1e-4) and np.allclose(pts[1], [60, 60], atol=1e-3)
    # centre from the first cubic's end points and the ellipse equation
    th = math.radians(rot)
    rot_inv = np.array([[math.cos(th), math.sin(th)], [-math.sin(th), math.cos(th)]])
    samples = []
    for x in c:
        P = np.array(unflip(x[2]), np.float64)
        for t in np.linspace(0, 1, 9):
            samples.append(((1 - t) ** 3) * P[0] + 3 * (1 - t) ** 2 * t * P[1] + 3 * (1 - t) * t * t * P[2] + t ** 3 * P[3])
    samples = np.array(samples)
    # fit the centre: points satisfy ((R^-1 (p - c)) / (rx, ry))^2 = 1
    from scipy.optimize import least_squares
    f = lambda cc: np.sum(((samples - cc) @ rot_inv.T / [rx, ry]) ** 2, axis=1) - 1
    res = least_squares(f, samples.mean(axis=0))
    assert np.abs(res.fun).max() < 2e-3
    # a zero radius is a straight line
    assert curves_of(one("M10 10 A0 5 0 0 1 20 20")) == [(0, L, unflip([[10, 10], [20, 20]]))]


def test_transforms():
    doc = ('<svg viewBox="0 0 100 100"><g transform="matrix(1,0,0,1,5,6) scale(2)">'
           '<g transform="translate(3)"><path d="M1 1 L2 1 L1 2 z" transform="rotate(45) scale(1 3)"/></g>'
           '</g></svg>')
    sc, _ = spr.Scene.parse_svg(doc)
    # (x, y) -> scale(1, 3) -> [rotate ignored] -> translate(3, 3) -> scale 2 -> +(5, 6)
    f = lambda x, y: [5 + 2 * (x + 3), 6 + 2 * (3 * y + 3)]
    assert curves_of(sc)[0][2] == unflip([f(1, 1), f(2, 1)])


def test_gradient_items():
    """The linear gradient's item maps x = 20..100 in the scene (10..90
    moved by the group's translate) to -1..1; its ramp runs red to blue at
    half alpha; the radial one is centred at (40, 40) of radius 30 in
    the flipped scene."""
    sc, _ = spr.Scene.parse_svg(DOC, srgb_ramps=False)
    table, ramp = sc.gradients
    t = table.view(np.float32).reshape(-1, 12)
    ti = table.view(np.int32).reshape(-1, 12)
    lin = t[1]
    gx = lambda x, y: lin[0] * x + lin[1] * y + lin[2]
    assert gx(20, 50) == pytest.approx(-1, abs=1e-5) and gx(100, 50) == pytest.approx(1, abs=1e-5)
    n = round(lin[7] * 1024) + 1
    r = ramp[ti[1, 6]:ti[1, 6] + n]
    assert r[0] == 0xFF0000FF and (r[-1] >> 24) == 127 and (r[-1] & 0xFFFFFF) in (0xFE0000, 0xFF0000)
    rad = t[4]
    cx = lambda x, y: (rad[0] * x + rad[1] * y + rad[2], rad[3] * x + rad[4] * y + rad[5])
    assert np.allclose(cx(40, 60), [0, 0], atol=1e-5) and np.allclose(cx(70, 60), [1, 0], atol=1e-5)
    assert np.allclose(cx(40, 30), [0, 1], atol=1e-5)  # y flipped: scene y 30 is SVG y 70


def test_oracle_renders_the_document():
    sc, info = spr.Scene.parse_svg(DOC, srgb_ramps=False)
    W, H = info["width"], info["height"]
    img = oracle.run(sc, W, H, samples=32, srgb=False)["IMAGE"].reshape(H, W, 4)
    # image rows are scene y; SVG y = H - scene y
    svg = lambda x, y: img[H - 1 - y, x].tolist()
    # green at alpha 127 over white (alpha blends too: 0.498^2 + 0.502 -> 191)
    assert svg(55, 10) == [128, 255, 128, 191]
    assert svg(125, 20) == [0x11, 0x22, 0x33, 255]        # polygon in its stroke colour
    assert svg(2, 2) == [255, 255, 255, 255]              # background
    row = np.array([svg(x, 20) for x in range(72, 99)])   # 5/8 of the way to blue .. blue at half alpha
    assert np.all(np.diff(row[:, 0]) <= 0) and np.all(np.diff(row[:, 2]) >= 0) and row[-1, 2] > row[0, 2]
    # radial about (40, 40): bluer outwards; its stops keep the stop-opacity
    # 0.5 of the linear gradient's last stop (the reference's current stop
    # carries over from stop to stop), so blue at half alpha over white
    near, far = svg(40, 61), svg(68, 93)
    assert near[0] > far[0] and near[1] > far[1] and near[2] < far[2] and far[:3] == [128, 128, 255]


def test_stroke_to_fill_flag():
    sc, info = spr.Scene.parse_svg(DOC, stroke_to_fill=True)
    assert info["n_paths"] == 6
    # the polygon keeps its own fill and is followed by its outline in #123
    assert sc.path_fill_rgba.tolist()[2:4] == [0xFF1E140A, 0xFF332211]
    assert sc.gradients is not None
    img = oracle.run(sc, 200, 100, samples=32)["IMAGE"].reshape(100, 200, 4)
    assert img[100 - 1 - 10, 125].tolist() == [0x11, 0x22, 0x33, 255]   # on the top edge's stroke
    assert img[100 - 1 - 25, 125].tolist() == [10, 20, 30, 255]         # inside: the fill


@pytest.mark.parametrize("doc,status", [
    ('<svg viewBox="0 0 9 9"><rect x="1" y="1" width="2" height="2"/></svg>', spr.ERR_UNSUPPORTED),
    ('<svg viewBox="0 0 9 9"><circle cx="1" cy="1" r="2"/></svg>', spr.ERR_UNSUPPORTED),
    ('<svg viewBox="0 0 9 9"><path d="M0 0 L1 1" fill="red"/></svg>', spr.ERR_UNSUPPORTED),
    ('<svg viewBox="0 0 9 9"><path d="M0 0 L1 1" fill="rgba(1,2,3,0.5)"/></svg>', spr.ERR_UNSUPPORTED),
    ('<svg viewBox="0 0 9 9"><path d="M0 0 L1 1 T2 2"/></svg>', spr.ERR_UNSUPPORTED),
    ('<svg viewBox="0 0 9 9"><path d="M0 0 L1 1" style="fill:#fff"/></svg>', spr.ERR_UNSUPPORTED),
    ('<svg viewBox="0 0 9 9"><path d="M0 0 L1 1" color="#fff"/></svg>', spr.ERR_UNSUPPORTED),
    ('<svg viewBox="0 0 9 9"><linearGradient id="a" gradientUnits="objectBoundingBox"/></svg>',
     spr.ERR_UNSUPPORTED),
    ('<svg viewBox="0 0 9 9"><path d="M0 0 L1 1" fill="url(#nope)"/></svg>', spr.ERR_INVALID_SCENE),
    ('<svg viewBox="0 0 9 9"><path d="M0 0 L1 1" transform="spin(3)"/></svg>', spr.ERR_INVALID_SCENE),
    ('<svg viewBox="0 0 9 9"><path d="M0 0 L1 1"></svg>', spr.ERR_INVALID_SCENE),
    ('<svg viewBox="0,0,9,9"><path d="M0 0 L1 1"/></svg>', spr.ERR_INVALID_SCENE),
    ('<svg><path d="M0 0 L1 1"/></svg>', spr.ERR_INVALID_SCENE),
])
def test_documents_the_reference_cannot_read(doc, status):
    with pytest.raises(spr.SprError) as e:
        spr.Scene.parse_svg(doc)
    assert e.value.status == status


def test_load_file_and_size_fallback(tmp_path):
    f = tmp_path / "doc.svg"
    f.write_text(DOC)
    a, ia = spr.Scene.load_svg(f)
    b, ib = spr.Scene.parse_svg(DOC)
    assert ia == ib and np.array_equal(a.vertex, b.vertex)
    with pytest.raises(spr.SprError) as e:
        spr.Scene.load_svg(tmp_path / "missing.svg")
    assert e.value.status == spr.ERR_INVALID_ARG
    sc, info = spr.Scene.parse_svg('<svg width="40px" height="30"><path d="M0 0 L10 0 L0 10 z"/></svg>')
    assert (info["width"], info["height"]) == (40, 30) and curves_of(sc)[0][2] == [[0, 30], [10, 30]]
    # a path element without d adds nothing; unknown elements are skipped with their children
    sc, info = spr.Scene.parse_svg('<svg viewBox="0 0 9 9"><path fill="#fff"/><x><path d="M0 0 L1 1"/></x></svg>')
    assert info["n_paths"] == 0 and sc.n_curves == 0


@pytest.mark.gpu
@pytest.mark.parametrize("stroke", [False, True])
def test_gpu_parity_on_a_loaded_svg(stroke):
    sc, info = spr.Scene.parse_svg(DOC, stroke_to_fill=stroke)
    W, H = info["width"], info["height"]
    for samples in (8, 32):
        ref = oracle.run(sc, W, H, samples=samples)["IMAGE"]
        with spr.VGRasterizer(W, H, samples=samples) as r:
            r.add_vg(sc)
            r.rasterize()
            assert np.array_equal(r.read_image().reshape(-1), ref), samples
