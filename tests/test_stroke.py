"""Stroke-to-fill (spr_stroke_to_fill, after VGContainer::strokeToOffsetCurve
and SimpleBezierCurve::segApproxOffsetCurve): outline structure, closure,
offset accuracy against the exact offset curve in float64, the fill/stroke
path bookkeeping, and renders of stroked scenes."""
import ctypes as C

import numpy as np
import pytest

import oracle
import spr

L, Q, CU, R = spr.CURVE_LINEAR, spr.CURVE_QUADRATIC, spr.CURVE_CUBIC, spr.CURVE_RATIONAL
RED = 0xFF0000FF


def one_path(curves, fill=0, rule=0):
    """A one-path scene from (type, points[, w]) tuples."""
    verts, pos, types, ws = [], [], [], []
    for c in curves:
        pos.append(len(verts))
        types.append(c[0])
        verts += [tuple(p) for p in c[1]]
        ws.append(c[2] if c[0] == R else -1.0)
    n = len(curves)
    return spr.Scene(np.array(verts, np.float32), [0] * len(verts), pos, types, [0] * n, ws, [rule], [fill])


def curves_of(sc, path=None):
    out = []
    for c in range(sc.n_curves):
        if path is not None and sc.curve_path_id[c] != path:
            continue
        p0, n = sc.curve_vertex_pos[c], sc.curve_type[c] & 7
        out.append((int(sc.curve_type[c]), sc.vertex[p0:p0 + n].astype(np.float64), float(sc.curve_arc_w[c])))
    return out


def loops(curves):
    """Splits a curve list into contours (a curve whose first point differs
    from the previous one's last starts a contour); checks each is closed."""
    out = []
    for c in curves:
        if not out or not np.array_equal(c[1][0], out[-1][-1][1][-1]):
            out.append([])
        out[-1].append(c)
    for lp in out:
        assert np.array_equal(lp[0][1][0], lp[-1][1][-1]), "open outline"
    return out


def exact_point(c, t):
    """float64 point of a scene curve (rational middle point stored
    Euclidean, homogeneous = point x w)."""
    kind, P, w = c
    t = np.asarray(t, np.float64)[:, None]
    u = 1 - t
    if kind == L:
        return u * P[0] + t * P[1]
    if kind == Q:
        return u * u * P[0] + 2 * u * t * P[1] + t * t * P[2]
    if kind == CU:
        return u ** 3 * P[0] + 3 * u * u * t * P[1] + 3 * u * t * t * P[2] + t ** 3 * P[3]
    num = u * u * P[0] + 2 * u * t * w * P[1] + t * t * P[2]
    return num / (u * u + 2 * u * t * w + t * t)


def exact_offset(c, h, n=20001):
    t = np.linspace(0, 1, n)
    p = exact_point(c, t)
    d = np.gradient(p, t, axis=0)
    nrm = np.stack([d[:, 1], -d[:, 0]], 1) / np.linalg.norm(d, axis=1)[:, None]
    return p + h * nrm


def dist_to_polyline(q, poly):
    """Distance of each point of q to the polyline poly."""
    a, b = poly[:-1], poly[1:]
    ab = b - a
    out = np.empty(len(q))
    for i, x in enumerate(q):
        s = np.clip(np.einsum("ij,ij->i", x - a, ab) / np.maximum(np.einsum("ij,ij->i", ab, ab), 1e-300), 0, 1)
        out[i] = np.min(np.linalg.norm(a + s[:, None] * ab - x, axis=1))
    return out


def test_line_stroke_is_a_rectangle():
    """Butt caps: a horizontal line of width 4 becomes the rectangle around
    it, drawn cap, positive side, cap, negative side; it renders exactly as
    that rectangle filled."""
    sc = one_path([(L, [(10, 20), (50, 20)])])
    out, info = sc.stroke_to_fill(RED, 4.0)
    assert info == {"n_fill_paths": 0, "n_stroke_paths": 1, "n_offset_pieces": 2, "max_depth": 0}
    assert out.curve_type.tolist() == [L] * 4 and out.path_fill_rgba.tolist() == [RED]
    assert out.path_fill_rule.tolist() == [0]
    assert out.vertex.tolist() == [[10, 22], [10, 18], [10, 18], [50, 18], [50, 18], [50, 22], [50, 22], [10, 22]]
    rect = one_path([(L, [(10, 22), (10, 18)]), (L, [(10, 18), (50, 18)]), (L, [(50, 18), (50, 22)]),
                     (L, [(50, 22), (10, 22)])], fill=RED)
    a = oracle.run(out, 64, 48, samples=32)["IMAGE"]
    b = oracle.run(rect, 64, 48, samples=32)["IMAGE"]
    assert np.array_equal(a, b)


def test_bevel_joins_and_fill_path():
    """An L of two lines, filled and stroked: the fill path first (the open
    contour closed by a line), then the outline with a bevel line at the
    corner on each side."""
    sc = one_path([(L, [(10, 20), (50, 20)]), (L, [(50, 20), (50, 60)])], fill=0xFF00FF00, rule=1)
    out, info = sc.stroke_to_fill(RED, 4.0)
    assert (info["n_fill_paths"], info["n_stroke_paths"]) == (1, 1)
    assert out.path_fill_rgba.tolist() == [0xFF00FF00, RED] and out.path_fill_rule.tolist() == [1, 0]
    fill = curves_of(out, 0)
    assert [c[1].tolist() for c in fill] == [[[10, 20], [50, 20]], [[50, 20], [50, 60]], [[50, 60], [10, 20]]]
    st = curves_of(out, 1)
    assert [c[1].tolist() for c in st] == [
        [[10, 22], [10, 18]], [[10, 18], [50, 18]], [[50, 18], [52, 20]],   # cap, side, bevel
        [[52, 20], [52, 60]], [[52, 60], [48, 60]],                          # side, end cap
        [[48, 60], [48, 20]], [[48, 20], [50, 22]], [[50, 22], [10, 22]]]    # back, bevel, back
    assert len(loops(st)) == 1


@pytest.mark.parametrize("curve", [
    (Q, [(10, 80), (80, 0), (150, 80)]),
    (CU, [(10, 100), (60, 20), (140, 180), (190, 100)]),
    (CU, [(10, 10), (10, 10), (120, 40), (150, 150)]),     # first control point doubled
    (CU, [(10, 10), (90, 10), (90, 10), (150, 150)]),      # middle control points equal
    (R, [(20, 100), (100, 20), (180, 100)], 0.7071067690849304),
    (R, [(20, 100), (100, 60), (180, 100)], 2.0),
])
@pytest.mark.parametrize("width", [2.0, 9.0])
def test_offset_accuracy(curve, width):
    """Every offset piece lies within 1/32 px of the exact offset curve
    (float64), the pieces cover it, and the outline closes."""
    c = (curve[0], np.array(curve[1], np.float64), curve[2] if len(curve) > 2 else -1.0)
    sc = one_path([curve])
    out, info = sc.stroke_to_fill(RED, width)
    assert 1 <= info["max_depth"] <= 8
    st = curves_of(out)
    assert len(loops(st)) == 1
    h = width / 2
    pos, neg = exact_offset(c, h), exact_offset(c, -h)
    n_side = (len(st) - 2) // 2
    t = np.linspace(0, 1, 9)
    for side, (ref, group) in enumerate(((pos, st[1:1 + n_side]), (neg, st[2 + n_side:]))):
        pts = np.concatenate([exact_point(p, t) for p in group])
        assert dist_to_polyline(pts, ref).max() < 1 / 32, side
        # the exact offset is covered by the pieces
        approx = np.concatenate([exact_point(p, np.linspace(0, 1, 65)) for p in group])
        assert dist_to_polyline(ref[::400], approx).max() < 1 / 32, side


def test_contours_affines_and_skipped_paths():
    """Two contours in one path give two outlines; a per-path affine is kept
    on both paths of its input path; a path with no fill and no stroke, and
    widths <= 0, add nothing; fill values (gradient entries) pass through."""
    sq = lambda x, y, s: [(x, y), (x + s, y), (x + s, y), (x + s, y + s), (x + s, y + s), (x, y + s),
                          (x, y + s), (x, y)]
    v = sq(10, 10, 20) + sq(40, 10, 10) + sq(5, 40, 8) + sq(30, 40, 8)
    vp = [0] * 16 + [1] * 8 + [2] * 8
    cp = list(range(0, 32, 2))
    cpid = [0] * 8 + [1] * 4 + [2] * 4
    aff = np.array([[1, 0, 0, 1, 0, 0], [2, 0, 0, 2, 1, 1], [1, 0, 0, 1, 0, 0]], np.float32)
    sc = spr.Scene(np.array(v, np.float32), vp, cp, [L] * 16, cpid, [-1] * 16, [0, 0, 1], [5, 0, 0], aff)
    out, info = sc.stroke_to_fill([0xFF112233, 0xFF445566, 0xFF778899], [3.0, 1.5, 0.0])
    assert (info["n_fill_paths"], info["n_stroke_paths"]) == (1, 2)
    assert out.path_fill_rgba.tolist() == [5, 0xFF112233, 0xFF445566]
    assert out.path_fill_rule.tolist() == [0, 0, 0]
    assert np.array_equal(out.path_affine, aff[[0, 0, 1]])
    assert len(loops(curves_of(out, 1))) == 2 and len(loops(curves_of(out, 2))) == 1
    assert len(curves_of(out, 1)) == 2 * 16  # 4 n per contour of n lines
    assert np.array_equal(out.vertex_path_id, np.repeat(out.curve_path_id, out.curve_type & 7))
    assert spr.lib().spr_validate_scene(out.view()) == spr.OK


def test_closed_square_renders_a_band():
    sq = [(L, [(16, 16), (48, 16)]), (L, [(48, 16), (48, 48)]), (L, [(48, 48), (16, 48)]),
          (L, [(16, 48), (16, 16)])]
    out, _ = one_path(sq).stroke_to_fill(RED, 6.0)
    img = oracle.run(out, 64, 64, samples=32)["IMAGE"].reshape(64, 64, 4)
    assert img[32, 32].tolist() == [255, 255, 255, 255]      # inside the band: background
    assert img[4, 4].tolist() == [255, 255, 255, 255]        # outside
    for y, x in ((16, 32), (32, 47), (47, 32), (32, 16)):    # on the band
        assert img[y, x].tolist() == [255, 0, 0, 255], (y, x)


def test_generated_scene_outlines_close():
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=11, width=256, height=256, n_paths=24, with_rational=True)
    rng = np.random.default_rng(3)
    out, info = sc.stroke_to_fill(0xC0406080, rng.uniform(0.5, 8, sc.n_paths).astype(np.float32))
    assert info["n_stroke_paths"] == sc.n_paths and info["n_fill_paths"] == int(np.count_nonzero(sc.path_fill_rgba))
    assert np.all(np.isfinite(out.vertex))
    for p in range(out.n_paths):
        loops(curves_of(out, p))  # every contour closed
    assert spr.lib().spr_validate_scene(out.view()) == spr.OK


def test_errors():
    sc = one_path([(L, [(10, 20), (50, 20)])])
    with pytest.raises(spr.SprError) as e:
        sc.stroke_to_fill(RED, np.nan)
    assert e.value.status == spr.ERR_INVALID_ARG
    h, info = C.c_void_p(), spr.StrokeInfo()
    assert spr.lib().spr_stroke_to_fill(C.byref(sc.view()), None, C.byref(h), C.byref(info)) == spr.ERR_INVALID_ARG
    bad = spr.Scene(np.zeros((2, 2), np.float32), [0, 0], [1], [L], [0], [-1], [0], [RED])
    with pytest.raises(spr.SprError) as e:
        bad.stroke_to_fill(RED, 1.0)
    assert e.value.status == spr.ERR_INVALID_SCENE


@pytest.mark.gpu
@pytest.mark.parametrize("samples", [8, 32])
def test_gpu_parity_on_stroked_scenes(samples):
    """Stroked scenes (generated paths, per-path affines, a loaded document
    with gradient paints) bit-exact against the oracle."""
    from test_rvg import DOC
    rng = np.random.default_rng(5)
    cases = []
    for aff in (False, True):
        sc = spr.Scene.generate(spr.SCENE_MIXED, seed=21 + aff, width=320, height=256, n_paths=40,
                                with_rational=True, with_affine=aff)
        st, _ = sc.stroke_to_fill(rng.integers(1, 2 ** 32, sc.n_paths, dtype=np.uint32) | 0x80000000,
                                  rng.uniform(0.5, 10, sc.n_paths).astype(np.float32))
        cases.append((st, 320, 256))
    doc, info = spr.Scene.parse_rvg(DOC)
    st, _ = doc.stroke_to_fill(0xFF203040, 3.0)
    cases.append((st, info["width"], info["height"]))
    for sc, W, H in cases:
        ref = oracle.run(sc, W, H, samples=samples)["IMAGE"]
        with spr.VGRasterizer(W, H, samples=samples) as r:
            r.add_vg(sc)
            r.rasterize()
            assert np.array_equal(r.read_image().reshape(-1), ref)


def test_degenerate_curves():
    """Zero-length and collinear curves, coincident control points, huge and
    tiny widths: finite closed outlines (or an error status), never NaN."""
    rng = np.random.default_rng(31)
    kinds = [(L, 2), (Q, 3), (CU, 4), (R, 3)]
    for trial in range(200):
        curves = []
        p = rng.integers(0, 4, 2).astype(np.float32) * 5
        for _ in range(int(rng.integers(1, 5))):
            k, n = kinds[int(rng.integers(0, 4))]
            pts = [p] + [rng.integers(0, 4, 2).astype(np.float32) * 5 if rng.random() < 0.6 else p for _ in range(n - 1)]
            if rng.random() < 0.2:  # collinear
                d = rng.normal(size=2).astype(np.float32)
                pts = [p + d * t for t in np.linspace(0, 3, n).astype(np.float32)]
            curves.append((k, [tuple(map(float, q)) for q in pts], float(rng.uniform(0.2, 3))))
            p = np.asarray(pts[-1], np.float32)
        sc = one_path(curves)
        width = float([1e-3, 0.5, 4.0, 1e4][trial % 4])
        try:
            out, _ = sc.stroke_to_fill(RED, width)
        except spr.SprError as e:
            assert e.status == spr.ERR_INVALID_SCENE
            continue
        assert np.all(np.isfinite(out.vertex))
        loops(curves_of(out))
