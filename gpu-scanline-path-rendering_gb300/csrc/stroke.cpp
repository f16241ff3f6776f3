// stroke.cpp -- stroke-to-fill: stroked paths become nonzero fill paths that
// enter the same fill pipeline (spr_stroke_to_fill in include/spr.h).
//
// The outline is the one VGContainer::strokeToOffsetCurve builds
// (gpu-scanline/src/vg_container.cpp:555-1353) as its live code runs:
//   * per input path, the fill path first, each contour closed by a line when
//     its two ends differ (:570-652), then one nonzero stroke path (:656-673);
//   * per contour of the stroke path: a butt cap from the negative side to the
//     positive side at the start (:762-795; the cap switch is commented out, so
//     every cap is butt), the curves offset by +width/2 with a bevel line
//     between consecutive curves (:824-965; the join type is forced to bevel at
//     :900), the end cap (:970-1035), then the curves reversed and offset by
//     +width/2 -- the negative side -- in reverse order with bevel lines
//     (:1039-1182).
// Each offset curve becomes fill curves as SimpleBezierCurve::
// segApproxOffsetCurve does (gpu-scanline/src/bezier_curve.cpp:548-590):
// halving in t from depth 1; each piece is approximated by a curve of its own
// kind through the offset end points with inner control points on the end
// tangents (d_approxOffsetCurve, bezier_curve.h:840-1003); a piece is kept
// when its offset mid point lies within 1/32 px of the approximation's mid
// point, or at depth 8.
//
// Defined behaviours where the reference is unfinished:
//   * joins are indexed per contour (the reference indexes its per-contour
//     end-point arrays with the scene-wide curve index, vg_container.cpp:873
//     and :1097, which only lines up for the scene's first contour);
//   * the negative side's end points are taken on the reversed curves, the
//     same evaluations that start and end its pieces, so every outline closes
//     bit for bit (the reference takes them from the forward curve offset by
//     -width/2, which can differ in the last bit);
//   * rational curves are evaluated with their middle control point in
//     homogeneous form (stored point x weight), the form the scene arrays
//     hold it in (rvg.cpp:341-348 stores v_mid / w1); the reference's offset
//     helpers use the stored point as the homogeneous one and mis-group the
//     quotient rule (bezier_curve.h:334-371);
//   * a tangent shorter than 1/1024 is replaced by a widening central
//     difference, the cubic rule of bezier_curve.h:300-323, for every kind; a
//     zero or non-finite tangent gives a zero normal (the point itself);
//   * a failed tangent-line intersection (parallel lines: a zero or
//     non-finite solution) takes the device approximation's fallbacks: the
//     offset mid point for quadratics and rationals, a line for degenerate
//     cubics, the offset middle-leg end points for general cubics.
// Contours are not stored in the scene arrays: a curve starts a contour when
// it is its path's first or its first vertex differs from the previous
// curve's last.

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "spr_scene.h"

namespace {

struct V2 {
    float x, y;
};
V2 add(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
V2 sub(V2 a, V2 b) { return {a.x - b.x, a.y - b.y}; }
V2 mul(V2 a, float s) { return {a.x * s, a.y * s}; }
V2 lerp(V2 a, V2 b, float t) { return {a.x + t * (b.x - a.x), a.y + t * (b.y - a.y)}; }  // lerp2, cutil_math.h:1027
bool same(V2 a, V2 b) { return a.x == b.x && a.y == b.y; }
bool finite(V2 a) { return std::isfinite(a.x) && std::isfinite(a.y); }

// A curve of the scene arrays: v[1] of a rational is the stored (Euclidean)
// middle point, w its weight.
struct Bez {
    int type;
    V2 v[4];
    float w;
};

Bez reversed(const Bez &c) {
    Bez r = c;
    const int n = c.type & 7;
    for (int i = 0; i < n; ++i) r.v[i] = c.v[n - 1 - i];
    return r;
}

// bezier_curve_point (bezier_curve.h:59-92), de Casteljau form.
V2 point(const Bez &c, float t) {
    switch (c.type) {
    case SPR_CURVE_LINEAR:
        return lerp(c.v[0], c.v[1], t);
    case SPR_CURVE_QUADRATIC:
        return lerp(lerp(c.v[0], c.v[1], t), lerp(c.v[1], c.v[2], t), t);
    case SPR_CURVE_CUBIC: {
        const V2 q0 = lerp(c.v[0], c.v[1], t), q1 = lerp(c.v[1], c.v[2], t), q2 = lerp(c.v[2], c.v[3], t);
        return lerp(lerp(q0, q1, t), lerp(q1, q2, t), t);
    }
    default: {
        const V2 h = mul(c.v[1], c.w);
        const V2 q = lerp(lerp(c.v[0], h, t), lerp(h, c.v[2], t), t);
        const float u = 1.f - t;
        const float wt = u * u + 2.f * u * t * c.w + t * t;
        return wt != 0.f ? mul(q, 1.f / wt) : V2{0.f, 0.f};  // safeRcp, cutil_math.h:862
    }
    }
}

// The curve's derivative direction (bezier_curve_tangent, bezier_curve.h:154-214).
V2 tangent(const Bez &c, float t) {
    const float u = 1.f - t;
    V2 d;
    switch (c.type) {
    case SPR_CURVE_LINEAR:
        d = sub(c.v[1], c.v[0]);
        break;
    case SPR_CURVE_QUADRATIC:
        d = add(mul(sub(c.v[1], c.v[0]), 2 * u), mul(sub(c.v[2], c.v[1]), 2 * t));
        break;
    case SPR_CURVE_CUBIC:
        d = add(add(mul(sub(c.v[1], c.v[0]), 3 * u * u), mul(sub(c.v[2], c.v[1]), 6 * u * t)),
                mul(sub(c.v[3], c.v[2]), 3 * t * t));
        break;
    default: {  // q'(t) w(t) - q(t) w'(t): the quotient rule's numerator
        const V2 h = mul(c.v[1], c.w);
        const V2 q = add(add(mul(c.v[0], u * u), mul(h, 2 * t * u)), mul(c.v[2], t * t));
        const V2 dq = add(mul(sub(h, c.v[0]), 2 * u), mul(sub(c.v[2], h), 2 * t));
        const float wt = u * u + 2 * t * u * c.w + t * t;
        const float dwt = 2 * u * (c.w - 1) + 2 * t * (1 - c.w);
        d = sub(mul(dq, wt), mul(q, dwt));
        break;
    }
    }
    float len = std::sqrt(d.x * d.x + d.y * d.y);
    for (float dt = 1 / 1024.f; len < 1 / 1024.f && dt <= 1; dt *= 2.f) {
        const float t0 = t - dt < 0.f ? 0.f : t - dt, t1 = t + dt > 1.f ? 1.f : t + dt;
        d = sub(point(c, t1), point(c, t0));
        len = std::sqrt(d.x * d.x + d.y * d.y);
    }
    return d;
}

// offset_bezier_curve_point (bezier_curve.h:264-391): the point moved by
// `off` along the unit normal (dy, -dx) / |d|.
V2 offset_point(const Bez &c, float off, float t) {
    const V2 d = tangent(c, t);
    const float len = std::sqrt(d.x * d.x + d.y * d.y);
    V2 n{0.f, 0.f};
    if (len > 0.f && std::isfinite(len)) n = {d.y / len, -d.x / len};
    return add(point(c, t), mul(n, off));
}

// d_subcurve (bezier_curve.h:398-515): the piece [t0, t1] as a curve of the
// same kind.
Bez subcurve(const Bez &c, float t0, float t1) {
    Bez o = c;
    switch (c.type) {
    case SPR_CURVE_LINEAR:
        o.v[0] = lerp(c.v[0], c.v[1], t0);
        o.v[1] = lerp(c.v[0], c.v[1], t1);
        break;
    case SPR_CURVE_QUADRATIC: {
        const V2 a0 = lerp(c.v[0], c.v[1], t0), a1 = lerp(c.v[1], c.v[2], t0);
        const V2 b0 = lerp(c.v[0], c.v[1], t1), b1 = lerp(c.v[1], c.v[2], t1);
        o.v[0] = lerp(a0, a1, t0);
        o.v[1] = lerp(a0, a1, t1);
        o.v[2] = lerp(b0, b1, t1);
        break;
    }
    case SPR_CURVE_CUBIC: {
        // the left part up to t1, then its right part from t0 / t1
        const float a = t1;
        float b = t0 / t1;
        if (b != b) b = 0.f;
        V2 c30 = lerp(c.v[0], c.v[1], a), c31 = lerp(c.v[1], c.v[2], a), c32 = lerp(c.v[2], c.v[3], a);
        V2 c20 = lerp(c30, c31, a), c21 = lerp(c31, c32, a);
        const V2 l0 = c.v[0], l1 = c30, l2 = c20, l3 = lerp(c20, c21, a);
        c30 = lerp(l0, l1, b);
        c31 = lerp(l1, l2, b);
        c32 = lerp(l2, l3, b);
        c20 = lerp(c30, c31, b);
        c21 = lerp(c31, c32, b);
        o.v[0] = lerp(c20, c21, b);
        o.v[1] = c21;
        o.v[2] = c32;
        o.v[3] = l3;
        break;
    }
    default: {
        // blossoms of the homogeneous curve; end weights renormalised to 1
        const V2 h = mul(c.v[1], c.w);
        auto blossom = [&](float s, float t, float &w) {
            const float st = s * t, b0 = st - s - t + 1, b1 = s + t - 2 * st, b2 = st;
            w = b0 + c.w * b1 + b2;
            return add(add(mul(c.v[0], b0), mul(h, b1)), mul(c.v[2], b2));
        };
        float wa, wb, wc;
        const V2 A = blossom(t0, t0, wa), B = blossom(t0, t1, wb), C = blossom(t1, t1, wc);
        const float s = 1.0f / std::sqrt(wa * wc);
        o.v[0] = t0 == 0.f ? c.v[0] : mul(A, 1.f / wa);
        o.v[2] = t1 == 1.f ? c.v[2] : mul(C, 1.f / wc);
        o.v[1] = mul(B, 1.f / wb);
        o.w = s * wb;
        break;
    }
    }
    return o;
}

// The point where the line p0 + a d0 meets the line p2 + b d2, by the 2x2
// inverse (solve_intersection, bezier_curve.cpp:372-395); false when the
// lines are parallel or the solution is not finite.
bool intersect(V2 p0, V2 d0, V2 p2, V2 d2, V2 &out) {
    const float ood = 1.f / (d0.x * d2.y - d2.x * d0.y);
    const V2 y = sub(p2, p0);
    const float a = (d2.y * ood) * y.x + (-d2.x * ood) * y.y;
    const float b = (-d0.y * ood) * y.x + (d0.x * ood) * y.y;
    if (!std::isfinite(a) || !std::isfinite(b)) return false;
    out = add(p0, mul(d0, a));
    return finite(out);
}

// d_approxOffsetCurve (bezier_curve.h:840-1003): a curve through the offset
// end points vf, vl approximating the piece c offset by `off`.
Bez approx(const Bez &c, float off, V2 vf, V2 vl) {
    Bez o = c;
    auto line = [&]() {
        o.type = SPR_CURVE_LINEAR;
        o.v[0] = vf;
        o.v[1] = vl;
    };
    switch (c.type) {
    case SPR_CURVE_LINEAR:
        line();
        break;
    case SPR_CURVE_QUADRATIC:
    case SPR_CURVE_RATIONAL: {
        V2 p1;
        if (!intersect(vf, sub(c.v[1], c.v[0]), vl, sub(c.v[1], c.v[2]), p1)) p1 = offset_point(c, off, .5f);
        o.v[0] = vf;
        o.v[1] = p1;
        o.v[2] = vl;
        break;
    }
    default: {
        const V2 *v = c.v;
        V2 p1, p2;
        if (same(v[0], v[1])) {
            if (!intersect(vf, sub(v[2], v[1]), vl, sub(v[2], v[3]), p1)) { line(); break; }
            o.v[0] = vf, o.v[1] = vf, o.v[2] = p1, o.v[3] = vl;
        } else if (same(v[1], v[2])) {
            if (!intersect(vf, sub(v[1], v[0]), vl, sub(v[2], v[3]), p1)) { line(); break; }
            o.v[0] = vf, o.v[1] = p1, o.v[2] = p1, o.v[3] = vl;
        } else if (same(v[2], v[3])) {
            if (!intersect(vf, sub(v[1], v[0]), vl, sub(v[1], v[3]), p1)) { line(); break; }
            o.v[0] = vf, o.v[1] = p1, o.v[2] = vl, o.v[3] = vl;
        } else {
            // the middle leg v1-v2 offset as a line; the end tangents meet it
            const Bez mid{SPR_CURVE_LINEAR, {v[1], v[2]}, -1.f};
            const V2 m1 = offset_point(mid, off, 0.f), m2 = offset_point(mid, off, 1.f);
            if (!intersect(vf, sub(v[1], v[0]), m2, sub(m1, m2), p1)) p1 = m1;
            if (!intersect(vl, sub(v[2], v[3]), m1, sub(m2, m1), p2)) p2 = m2;
            o.v[0] = vf, o.v[1] = p1, o.v[2] = p2, o.v[3] = vl;
        }
        break;
    }
    }
    return o;
}

constexpr float kTolerance = 1 / 32.f;
constexpr int kMaxDepth = 8;

struct Out {
    spr_scene *s;
    uint32_t path;
    uint32_t pieces = 0;
    int max_depth = 0;
    void curve(const Bez &c) {
        float xy[8];
        for (int i = 0; i < (c.type & 7); ++i) xy[2 * i] = c.v[i].x, xy[2 * i + 1] = c.v[i].y;
        s->add_curve(path, c.type, xy, c.w);
    }
    void line(V2 a, V2 b) { curve(Bez{SPR_CURVE_LINEAR, {a, b}, -1.f}); }
};

// segApproxOffsetCurve: the curve c offset by `off` as fill curves.
void offset_curve(const Bez &c, float off, Out &out) {
    if (c.type == SPR_CURVE_LINEAR) {
        out.curve(approx(c, off, offset_point(c, off, 0.f), offset_point(c, off, 1.f)));
        ++out.pieces;
        return;
    }
    struct Node {
        float l, r;
        int depth;
    };
    Node stack[kMaxDepth + 1];
    int top = 0;
    stack[top++] = {0.f, 1.f, 1};
    while (top) {  // depth first, left half before right half
        const Node nd = stack[--top];
        if (nd.depth > out.max_depth) out.max_depth = nd.depth;
        const Bez piece = subcurve(c, nd.l, nd.r);
        const Bez a = approx(piece, off, offset_point(c, off, nd.l), offset_point(c, off, nd.r));
        const V2 d = sub(offset_point(piece, off, .5f), point(a, .5f));
        if (std::sqrt(d.x * d.x + d.y * d.y) < kTolerance || nd.depth >= kMaxDepth) {
            out.curve(a);
            ++out.pieces;
            continue;
        }
        const float m = (nd.l + nd.r) * .5f;
        stack[top++] = {m, nd.r, nd.depth + 1};
        stack[top++] = {nd.l, m, nd.depth + 1};
    }
}

// The outline of one contour (curves c[0..n)) stroked with half width h.
void stroke_contour(const std::vector<Bez> &c, float h, Out &out) {
    const size_t n = c.size();
    std::vector<Bez> rev(n);
    std::vector<V2> p0(n), p1(n), n0(n), n1(n);  // positive / negative side at each curve's start / end
    for (size_t k = 0; k < n; ++k) {
        rev[k] = reversed(c[k]);
        p0[k] = offset_point(c[k], h, 0.f);
        p1[k] = offset_point(c[k], h, 1.f);
        n0[k] = offset_point(rev[k], h, 1.f);
        n1[k] = offset_point(rev[k], h, 0.f);
    }
    out.line(n0[0], p0[0]);
    for (size_t k = 0; k < n; ++k) {
        offset_curve(c[k], h, out);
        if (k + 1 < n) out.line(p1[k], p0[k + 1]);
    }
    out.line(p1[n - 1], n1[n - 1]);
    for (size_t k = n; k-- > 0;) {
        offset_curve(rev[k], h, out);
        if (k > 0) out.line(n0[k], n1[k - 1]);
    }
}

Bez curve_of(const spr_scene_view *v, uint32_t i) {
    Bez b{};
    b.type = v->curve_type[i];
    const uint32_t p = v->curve_vertex_pos[i];
    for (int k = 0; k < (b.type & 7); ++k) b.v[k] = {v->vertex[2 * (size_t)(p + k)], v->vertex[2 * (size_t)(p + k) + 1]};
    b.w = v->curve_arc_w ? v->curve_arc_w[i] : -1.f;
    return b;
}

V2 first_of(const Bez &b) { return b.v[0]; }
V2 last_of(const Bez &b) { return b.v[(b.type & 7) - 1]; }

}  // namespace

extern "C" int spr_stroke_to_fill(const spr_scene_view *in, const spr_stroke_style *styles, spr_scene **out,
                                  spr_stroke_info *info) {
    if (!in || !out || (!styles && in->n_paths)) return SPR_ERR_INVALID_ARG;
    *out = nullptr;
    const int st = spr_validate_scene(in);
    if (st) return st;
    for (uint32_t p = 0; p < in->n_paths; ++p)
        if (!std::isfinite(styles[p].width)) return SPR_ERR_INVALID_ARG;
    spr_scene *s = new (std::nothrow) spr_scene();
    if (!s) return SPR_ERR_OUT_OF_MEMORY;
    spr_stroke_info inf{};
    Out o{s, 0};
    try {
        uint32_t c = 0;
        for (uint32_t p = 0; p < in->n_paths; ++p) {
            const uint32_t c0 = c;
            while (c < in->n_curves && in->curve_path_id[c] == p) ++c;
            // contours of this path
            std::vector<std::vector<Bez>> contours;
            for (uint32_t i = c0; i < c; ++i) {
                const Bez b = curve_of(in, i);
                if (contours.empty() || !same(first_of(b), last_of(contours.back().back()))) contours.emplace_back();
                contours.back().push_back(b);
            }
            auto new_path = [&](uint8_t rule, uint32_t rgba) {
                o.path = (uint32_t)s->fill_rule.size();
                s->fill_rule.push_back(rule);
                s->fill_rgba.push_back(rgba);
                if (in->path_affine) s->affine.insert(s->affine.end(), in->path_affine + 6 * (size_t)p,
                                                      in->path_affine + 6 * (size_t)p + 6);
            };
            if (in->path_fill_rgba[p]) {
                new_path(in->path_fill_rule[p], in->path_fill_rgba[p]);
                ++inf.n_fill_paths;
                for (const auto &ct : contours) {
                    for (const Bez &b : ct) o.curve(b);
                    if (!same(first_of(ct.front()), last_of(ct.back()))) o.line(last_of(ct.back()), first_of(ct.front()));
                }
            }
            if (styles[p].rgba && styles[p].width > 0.f) {
                new_path(0, styles[p].rgba);  // nonzero (vg_container.cpp:669)
                ++inf.n_stroke_paths;
                for (const auto &ct : contours) stroke_contour(ct, styles[p].width * .5f, o);
            }
        }
    } catch (const std::bad_alloc &) {
        delete s;
        return SPR_ERR_OUT_OF_MEMORY;
    }
    s->has_affine = in->path_affine != nullptr;
    for (float x : s->vertex)
        if (!std::isfinite(x)) {
            delete s;
            return SPR_ERR_INVALID_SCENE;
        }
    inf.n_offset_pieces = o.pieces;
    inf.max_depth = o.max_depth;
    if (info) *info = inf;
    *out = s;
    return SPR_OK;
}
