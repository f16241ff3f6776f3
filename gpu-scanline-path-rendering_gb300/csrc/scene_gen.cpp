// scene_gen.cpp -- seeded synthetic scenes in the reference's flat scene
// layout (VGInputCurveDataPack / VGInputPathDataPack, ras_base.h:34-112).
//
// The reference benchmarks on MPVG .rvg documents that are not available
// here; these generators produce scenes of the same shape (closed paths of
// line / quadratic / cubic / rational segments, solid RGBA fills, both fill
// rules) from one 64-bit seed.  All geometry is computed in double and stored
// as float.  The random stream is xoshiro256** seeded by splitmix64, so a
// (spec, seed) pair gives bit-identical scenes on every host.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/spr.h"
#include "spr_scene.h"

namespace {

struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t z = seed;
        for (int i = 0; i < 4; ++i) {
            z += 0x9E3779B97F4A7C15ull;
            uint64_t x = z;
            x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
            x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
            s[i] = x ^ (x >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        uint64_t r = rotl(s[1] * 5, 7) * 9;
        uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
    int range(int lo, int hi) { return lo + (int)(uniform() * (double)(hi - lo + 1)); }  // [lo,hi]
};

struct P2 {
    double x, y;
};

}  // namespace

namespace {

void add_curve(spr_scene &s, uint32_t path, int type, const P2 *pts, double w) {
    float xy[8];
    for (int i = 0; i < (type & 7); ++i) {
        xy[2 * i] = (float)pts[i].x;
        xy[2 * i + 1] = (float)pts[i].y;
    }
    s.add_curve(path, type, xy, (float)w);
}

uint32_t add_path(spr_scene &s, Rng &rng) {
    uint32_t id = (uint32_t)s.fill_rule.size();
    uint32_t r = (uint32_t)std::lround(rng.uniform() * 255.0);
    uint32_t g = (uint32_t)std::lround(rng.uniform() * 255.0);
    uint32_t b = (uint32_t)std::lround(rng.uniform() * 255.0);
    uint32_t a = (uint32_t)std::lround(rng.uniform(0.5, 1.0) * 255.0);
    uint32_t c = r | (g << 8) | (b << 16) | (a << 24);
    s.fill_rgba.push_back((c & 0xFF000000u) ? c : 0u);
    s.fill_rule.push_back(rng.uniform() < 0.5 ? SPR_FILL_NONZERO : SPR_FILL_EVEN_ODD);
    return id;
}

}  // namespace

namespace {

// Curve type for a segment: 40% line, 30% quadratic, 30% cubic; with
// `rational`, a tenth of the quadratics become rational quadratics.
int pick_type(Rng &rng, bool rational, bool no_line) {
    double u = rng.uniform();
    if (no_line) u = 0.4 + 0.6 * u;
    if (u < 0.4) return SPR_CURVE_LINEAR;
    if (u < 0.7) {
        if (rational && rng.uniform() < 0.1) return SPR_CURVE_RATIONAL;
        return SPR_CURVE_QUADRATIC;
    }
    return SPR_CURVE_CUBIC;
}

// Closed contour through `pts` (cyclic): segment k runs pts[k] -> pts[k+1];
// interior control points come from `ctrl(k, j)`.  Endpoints are shared
// bit-exactly between consecutive segments.
template <class Ctrl>
void closed_contour(spr_scene &s, Rng &rng, uint32_t path, const std::vector<P2> &pts, bool rational,
                    bool no_line, bool cubic_only, Ctrl ctrl) {
    const size_t n = pts.size();
    for (size_t k = 0; k < n; ++k) {
        P2 a = pts[k], b = pts[(k + 1) % n];
        int type = cubic_only ? SPR_CURVE_CUBIC : pick_type(rng, rational, no_line);
        P2 cp[4];
        cp[0] = a;
        double w = 1.0;
        switch (type) {
        case SPR_CURVE_LINEAR:
            cp[1] = b;
            break;
        case SPR_CURVE_QUADRATIC:
            cp[1] = ctrl(a, b, 0.5);
            cp[2] = b;
            break;
        case SPR_CURVE_RATIONAL:
            cp[1] = ctrl(a, b, 0.5);
            cp[2] = b;
            w = rng.uniform(0.25, 2.0);
            break;
        default:
            cp[1] = ctrl(a, b, 1.0 / 3.0);
            cp[2] = ctrl(a, b, 2.0 / 3.0);
            cp[3] = b;
            break;
        }
        add_curve(s, path, type, cp, w);
    }
}

void gen_random(spr_scene &s, Rng &rng, const spr_scene_spec &sp) {
    const double W = sp.width, H = sp.height;
    auto rnd_pt = [&]() { return P2{rng.uniform(0.0, W), rng.uniform(0.0, H)}; };
    for (int p = 0; p < sp.n_paths; ++p) {
        uint32_t id = add_path(s, rng);
        int n = rng.range(sp.seg_min, sp.seg_max);
        std::vector<P2> pts(n);
        for (auto &q : pts) q = rnd_pt();
        closed_contour(s, rng, id, pts, sp.with_rational != 0, false, false,
                       [&](P2, P2, double) { return rnd_pt(); });
    }
}

// Like gen_random, with each path confined to its own random square box.
void gen_local(spr_scene &s, Rng &rng, const spr_scene_spec &sp) {
    const double W = sp.width, H = sp.height;
    const double dim = std::fmin(W, H);
    for (int p = 0; p < sp.n_paths; ++p) {
        uint32_t id = add_path(s, rng);
        const double side = rng.uniform(dim / 32.0, dim / 4.0);
        const double x0 = rng.uniform(-side * 0.5, W - side * 0.5), y0 = rng.uniform(-side * 0.5, H - side * 0.5);
        auto rnd_pt = [&]() { return P2{x0 + rng.uniform(0.0, side), y0 + rng.uniform(0.0, side)}; };
        int n = rng.range(sp.seg_min, sp.seg_max);
        std::vector<P2> pts(n);
        for (auto &q : pts) q = rnd_pt();
        closed_contour(s, rng, id, pts, sp.with_rational != 0, false, false,
                       [&](P2, P2, double) { return rnd_pt(); });
    }
}

// Star-shaped closed loop around the origin: n vertices at radius
// r * U[rlo, 1], angles jittered; control points offset from the chord.
std::vector<P2> star(Rng &rng, int n, double r, double rlo) {
    std::vector<P2> pts(n);
    for (int k = 0; k < n; ++k) {
        double th = 2.0 * M_PI * (k + rng.uniform(-0.3, 0.3)) / n;
        double rr = r * rng.uniform(rlo, 1.0);
        pts[k] = P2{rr * std::cos(th), rr * std::sin(th)};
    }
    return pts;
}

void gen_mixed(spr_scene &s, Rng &rng, const spr_scene_spec &sp) {
    const double W = sp.width, H = sp.height;
    const double dim = std::fmin(W, H);
    // Glyph-like paths: 10-40 quadratic/cubic segments in an 8-64 px box,
    // placed by a random affine (scale 0.5-4, any rotation).
    const int n_glyph = sp.n_paths;
    const int n_large = sp.n_large;
    // Interleave glyphs and large paths in painter's order.
    const int total = n_glyph + n_large;
    int g_left = n_glyph, l_left = n_large;
    for (int p = 0; p < total; ++p) {
        bool large = rng.uniform() * (g_left + l_left) < l_left;
        if (large) --l_left; else --g_left;
        uint32_t id = add_path(s, rng);
        if (!large) {
            double size = rng.uniform(8.0, 64.0);
            int n = rng.range(10, 40);
            std::vector<P2> pts = star(rng, n, size * 0.5, 0.45);
            double sc = rng.uniform(0.5, 4.0), th = rng.uniform(0.0, 2.0 * M_PI);
            double cx = rng.uniform(0.0, W), cy = rng.uniform(0.0, H);
            double a = sc * std::cos(th), b = sc * std::sin(th), c = -sc * std::sin(th), d = sc * std::cos(th);
            auto ctrl = [&](P2 u, P2 v, double f) {
                double jx = rng.uniform(-0.25, 0.25) * size, jy = rng.uniform(-0.25, 0.25) * size;
                return P2{u.x + (v.x - u.x) * f + jx, u.y + (v.y - u.y) * f + jy};
            };
            size_t first = s.curve_type.size();
            closed_contour(s, rng, id, pts, sp.with_rational != 0, true, false, ctrl);
            if (sp.with_affine) {
                s.affine.insert(s.affine.end(), {(float)a, (float)b, (float)c, (float)d, (float)cx, (float)cy});
            } else {
                // bake the affine into the vertices (as the reference's RVG loader does)
                for (size_t ci = first; ci < s.curve_type.size(); ++ci) {
                    uint32_t vp = s.curve_vertex_pos[ci];
                    for (int j = 0; j < (s.curve_type[ci] & 7); ++j) {
                        double x = s.vertex[2 * (vp + j)], y = s.vertex[2 * (vp + j) + 1];
                        s.vertex[2 * (vp + j)] = (float)(a * x + c * y + cx);
                        s.vertex[2 * (vp + j) + 1] = (float)(b * x + d * y + cy);
                    }
                }
            }
        } else {
            // Large path: a closed thin band around a random walk that spans
            // up to the whole viewport; 50-500 segments in total.
            int nseg = rng.range(50, 500);
            int m = std::max(2, nseg / 2 - 1);
            double hw = rng.uniform(1.0, 5.0);
            double len = rng.uniform(0.25, 1.25) * dim;
            double step = len / m;
            std::vector<P2> q(m + 1);
            q[0] = P2{rng.uniform(0.0, W), rng.uniform(0.0, H)};
            double phi = rng.uniform(0.0, 2.0 * M_PI);
            for (int k = 1; k <= m; ++k) {
                phi += rng.uniform(-0.5, 0.5);
                P2 nq{q[k - 1].x + step * std::cos(phi), q[k - 1].y + step * std::sin(phi)};
                if (nq.x < -0.05 * W || nq.x > 1.05 * W) {
                    phi = M_PI - phi;
                    nq.x = q[k - 1].x + step * std::cos(phi);
                }
                if (nq.y < -0.05 * H || nq.y > 1.05 * H) {
                    phi = -phi;
                    nq.y = q[k - 1].y + step * std::sin(phi);
                }
                q[k] = nq;
            }
            std::vector<P2> outline;
            outline.reserve(2 * (m + 1));
            auto normal = [&](int k) {
                P2 a = q[std::max(k - 1, 0)], b = q[std::min(k + 1, m)];
                double dx = b.x - a.x, dy = b.y - a.y, l = std::sqrt(dx * dx + dy * dy);
                if (l <= 0) return P2{0.0, 1.0};
                return P2{-dy / l, dx / l};
            };
            for (int k = 0; k <= m; ++k) {
                P2 nn = normal(k);
                outline.push_back(P2{q[k].x + hw * nn.x, q[k].y + hw * nn.y});
            }
            for (int k = m; k >= 0; --k) {
                P2 nn = normal(k);
                outline.push_back(P2{q[k].x - hw * nn.x, q[k].y - hw * nn.y});
            }
            auto ctrl = [&](P2 u, P2 v, double f) {
                double dx = v.x - u.x, dy = v.y - u.y, l = std::sqrt(dx * dx + dy * dy);
                double off = rng.uniform(-0.3, 0.3) * hw;
                double nx = l > 0 ? -dy / l : 0.0, ny = l > 0 ? dx / l : 0.0;
                return P2{u.x + dx * f + off * nx, u.y + dy * f + off * ny};
            };
            closed_contour(s, rng, id, outline, sp.with_rational != 0, false, false, ctrl);
            if (sp.with_affine) s.affine.insert(s.affine.end(), {1.f, 0.f, 0.f, 1.f, 0.f, 0.f});
        }
    }
    s.has_affine = sp.with_affine != 0;
}

void gen_cubics(spr_scene &s, Rng &rng, const spr_scene_spec &sp) {
    const double W = sp.width, H = sp.height, dim = std::fmin(W, H);
    for (int p = 0; p < sp.n_paths; ++p) {
        uint32_t id = add_path(s, rng);
        int n = rng.range(sp.seg_min, sp.seg_max);
        double r = rng.uniform(0.03, 0.25) * dim;
        std::vector<P2> pts = star(rng, n, r, 0.5);
        double cx = rng.uniform(0.0, W), cy = rng.uniform(0.0, H);
        for (auto &q : pts) q = P2{q.x + cx, q.y + cy};
        auto ctrl = [&](P2 u, P2 v, double f) {
            double jx = rng.uniform(-0.15, 0.15) * r, jy = rng.uniform(-0.15, 0.15) * r;
            return P2{u.x + (v.x - u.x) * f + jx, u.y + (v.y - u.y) * f + jy};
        };
        closed_contour(s, rng, id, pts, false, true, true, ctrl);
        if (sp.with_affine) s.affine.insert(s.affine.end(), {1.f, 0.f, 0.f, 1.f, 0.f, 0.f});
    }
    s.has_affine = sp.with_affine != 0;
}

}  // namespace

extern "C" int spr_scene_generate(const spr_scene_spec *spec, spr_scene **out) {
    if (!spec || !out) return SPR_ERR_INVALID_ARG;
    const spr_scene_spec &sp = *spec;
    if (sp.width < 1 || sp.height < 1 || sp.n_paths < 0 || sp.n_large < 0) return SPR_ERR_INVALID_ARG;
    if (sp.kind != SPR_SCENE_MIXED && (sp.seg_min < 1 || sp.seg_max < sp.seg_min)) return SPR_ERR_INVALID_ARG;
    spr_scene *s = new (std::nothrow) spr_scene();
    if (!s) return SPR_ERR_OUT_OF_MEMORY;
    Rng rng(sp.seed);
    switch (sp.kind) {
    case SPR_SCENE_RANDOM: gen_random(*s, rng, sp); break;
    case SPR_SCENE_MIXED: gen_mixed(*s, rng, sp); break;
    case SPR_SCENE_CUBICS: gen_cubics(*s, rng, sp); break;
    case SPR_SCENE_LOCAL: gen_local(*s, rng, sp); break;
    default: delete s; return SPR_ERR_INVALID_ARG;
    }
    if (sp.with_affine && (sp.kind == SPR_SCENE_RANDOM || sp.kind == SPR_SCENE_LOCAL)) {
        s->affine.clear();
        for (size_t p = 0; p < s->fill_rule.size(); ++p) s->affine.insert(s->affine.end(), {1.f, 0.f, 0.f, 1.f, 0.f, 0.f});
        s->has_affine = true;
    }
    *out = s;
    return SPR_OK;
}

extern "C" int spr_scene_view_of(const spr_scene *s, spr_scene_view *v) {
    if (!s || !v) return SPR_ERR_INVALID_ARG;
    v->n_paths = (uint32_t)s->fill_rule.size();
    v->n_curves = (uint32_t)s->curve_type.size();
    v->n_vertices = (uint32_t)(s->vertex.size() / 2);
    v->vertex = s->vertex.data();
    v->vertex_path_id = s->vertex_path_id.data();
    v->curve_vertex_pos = s->curve_vertex_pos.data();
    v->curve_type = s->curve_type.data();
    v->curve_path_id = s->curve_path_id.data();
    v->curve_arc_w = s->curve_arc_w.data();
    v->path_fill_rule = s->fill_rule.data();
    v->path_fill_rgba = s->fill_rgba.data();
    v->path_affine = s->has_affine ? s->affine.data() : nullptr;
    return SPR_OK;
}

extern "C" void spr_scene_free(spr_scene *s) { delete s; }
