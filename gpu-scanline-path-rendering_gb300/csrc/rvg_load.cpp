// rvg_load.cpp -- RVG documents (the MPVG text format the reference's
// benchmark reads) into a host scene, following RVG::load (rvg.cpp:62-776)
// and the fill conversion of VGRasterizer::addVg (ras_base.cpp:138-162).
//
// A document is a three-line header -- a keyword and two points (the
// viewport), a keyword and two points (the window), "scene dyn_identity" --
// then one element per line:
//
//   1 element <nzfill|ofill> dyn_concrete <p> <p> <p> <commands>
//     <dyn_identity|dyn_affine[[a,b,c],[d,e,f]]> dyn_paint <opacity>
//     <solid rgba(r,g,b,a)|solid rgb(r,g,b)|linear ...|radial ...>
//
// Points are "x,y" tokens (',' and ':' separate numbers).  Commands: M p
// (new contour), fL p (move), L p, Q p p, C p p p, A x,y,w p (rational arc;
// w = 0: a half circle of two quarter arcs), Z.  Every element that adds
// vertices becomes a path; an element that adds none leaves its path to the
// next one.  The last contour of an element is closed by a line when it was
// not closed by Z and ends away from its start.  Solid colours are
// truncated to 8 bits, alpha scaled by the opacity; colours with alpha 0
// become 0.  Linear and radial paints are counted and get the fill value
// path + 1 (the reference's gradient index, drawn by its gradient shader;
// here alpha 0, not drawn).  The reference's parsing quirks are kept: rgb()
// drops the last character of its third number, the three points after
// dyn_concrete are read and ignored.

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/spr.h"
#include "spr_scene.h"

namespace {

struct V2 {
    float x, y;
};

void separators_to_spaces(std::string &s) {
    for (char &c : s)
        if (c == ',' || c == ':') c = ' ';
}

bool read_point(std::istream &in, V2 &v) {
    std::string t;
    if (!(in >> t)) return false;
    separators_to_spaces(t);
    v = V2{0.f, 0.f};
    std::sscanf(t.c_str(), "%f %f", &v.x, &v.y);
    return true;
}

// (uint8_t)(x * 255) of frgba -> u8rgba (color.h), clamped where the
// truncation would leave 0..255.
uint32_t to_u8(float x) {
    const float v = x * 255.f;
    if (!(v > 0.f)) return 0u;
    if (v >= 255.f) return 255u;
    return (uint32_t)v;
}

struct Parser {
    std::istringstream in;
    spr_scene &sc;
    spr_rvg_info &info;
    bool a128;
    Parser(const std::string &text, spr_scene &s, spr_rvg_info &i, bool a) : in(text), sc(s), info(i), a128(a) {}

    uint32_t vertex_count() const { return (uint32_t)(sc.vertex.size() / 2); }
    V2 vertex(uint32_t i) const { return V2{sc.vertex[2 * i], sc.vertex[2 * i + 1]}; }

    void curve(uint32_t path, int type, const V2 *p, float w) {
        float xy[8];
        for (int i = 0; i < (type & 7); ++i) {
            xy[2 * i] = p[i].x;
            xy[2 * i + 1] = p[i].y;
        }
        sc.add_curve(path, type, xy, w);
    }

    void skip_line() {
        std::string rest;
        std::getline(in, rest);
    }

    int run() {
        std::string t;
        V2 vp[2], win[2];
        if (!(in >> t) || !read_point(in, vp[0]) || !read_point(in, vp[1])) return SPR_ERR_INVALID_SCENE;
        if (!(in >> t) || !read_point(in, win[0]) || !read_point(in, win[1])) return SPR_ERR_INVALID_SCENE;
        if (!(in >> t) || t != "scene" || !(in >> t) || t != "dyn_identity") return SPR_ERR_INVALID_SCENE;
        info.viewport[0] = vp[0].x;
        info.viewport[1] = vp[0].y;
        info.viewport[2] = vp[1].x;
        info.viewport[3] = vp[1].y;
        info.window[0] = win[0].x;
        info.window[1] = win[0].y;
        info.window[2] = win[1].x;
        info.window[3] = win[1].y;
        info.width = (int32_t)vp[1].x;
        info.height = (int32_t)vp[1].y;

        int64_t last_path_vertices = -1;
        uint32_t path = 0;
        while (in >> t) {
            if (t == "//") {
                skip_line();
                continue;
            }
            if (t != "1" || !(in >> t) || t != "element") return SPR_ERR_INVALID_SCENE;
            ++info.n_elements;
            if (last_path_vertices != (int64_t)vertex_count()) {  // a new path
                path = (uint32_t)sc.fill_rule.size();
                sc.fill_rule.push_back(SPR_FILL_NONZERO);
                sc.fill_rgba.push_back(0u);
                last_path_vertices = vertex_count();
            }
            std::string rule;
            if (!(in >> rule)) return SPR_ERR_INVALID_SCENE;
            if (rule == "nzfill") {
                sc.fill_rule[path] = SPR_FILL_NONZERO;
            } else if (rule == "ofill") {
                sc.fill_rule[path] = SPR_FILL_EVEN_ODD;
            } else {
                skip_line();
                continue;
            }
            if (!(in >> t)) return SPR_ERR_INVALID_SCENE;
            if (t == "depth") {
                skip_line();
                continue;
            }
            if (t != "dyn_concrete") return SPR_ERR_INVALID_SCENE;
            V2 p[4];
            for (int i = 0; i < 3; ++i)
                if (!read_point(in, p[i])) return SPR_ERR_INVALID_SCENE;
            const uint32_t path_begin = vertex_count();
            uint32_t contour_begin = path_begin;
            bool closed = false;
            while (in >> t) {
                if (t != "fL" && t.length() != 1) break;
                const char op = t[0];
                if (t != "fL" && std::string("MmZzLlHhVvCcSsQqTtAa").find(op) == std::string::npos) break;
                if (t == "fL") {
                    if (!read_point(in, p[0])) return SPR_ERR_INVALID_SCENE;
                    continue;
                }
                switch (op) {
                case 'M':
                    if (!read_point(in, p[0])) return SPR_ERR_INVALID_SCENE;
                    contour_begin = vertex_count();
                    closed = false;
                    break;
                case 'L':
                    if (!read_point(in, p[1])) return SPR_ERR_INVALID_SCENE;
                    curve(path, SPR_CURVE_LINEAR, p, 0.f);
                    p[0] = p[1];
                    break;
                case 'Q':
                    if (!read_point(in, p[1]) || !read_point(in, p[2])) return SPR_ERR_INVALID_SCENE;
                    curve(path, SPR_CURVE_QUADRATIC, p, 0.f);
                    p[0] = p[2];
                    break;
                case 'C':
                    if (!read_point(in, p[1]) || !read_point(in, p[2]) || !read_point(in, p[3]))
                        return SPR_ERR_INVALID_SCENE;
                    curve(path, SPR_CURVE_CUBIC, p, 0.f);
                    p[0] = p[3];
                    break;
                case 'A': {
                    std::string a;
                    if (!(in >> a)) return SPR_ERR_INVALID_SCENE;
                    separators_to_spaces(a);
                    V2 mid{0.f, 0.f};
                    float w = 0.f;
                    std::sscanf(a.c_str(), "%f %f %f", &mid.x, &mid.y, &w);
                    if (!(w >= 0.f || w <= 0.f)) w = 0.f;
                    if (!read_point(in, p[1])) return SPR_ERR_INVALID_SCENE;
                    if (w == 0.f) {
                        // half circle: mid is the direction of the arc's middle
                        // from the chord's centre; two quarter arcs
                        const V2 d{0.5f * (p[1].x - p[0].x), 0.5f * (p[1].y - p[0].y)};
                        const V2 m{0.5f * (p[0].x + p[1].x) + mid.x, 0.5f * (p[0].y + p[1].y) + mid.y};
                        const float qw = 0.7071067811865475244f;
                        const V2 a0[3] = {p[0], V2{m.x - d.x, m.y - d.y}, m};
                        const V2 a1[3] = {m, V2{m.x + d.x, m.y + d.y}, p[1]};
                        curve(path, SPR_CURVE_RATIONAL, a0, qw);
                        curve(path, SPR_CURVE_RATIONAL, a1, qw);
                    } else {
                        const V2 r[3] = {p[0], V2{mid.x / w, mid.y / w}, p[1]};
                        curve(path, SPR_CURVE_RATIONAL, r, w);
                    }
                    p[0] = p[1];
                    break;
                }
                case 'Z':
                    closed = true;
                    break;
                default:
                    return SPR_ERR_UNSUPPORTED;  // relative and shorthand commands
                }
            }
            if (!in) return SPR_ERR_INVALID_SCENE;
            if (vertex_count() == path_begin) {  // nothing drawn: the path waits for the next element
                skip_line();
                continue;
            }
            if (!closed && vertex_count() > contour_begin) {
                const V2 first = vertex(contour_begin), last = vertex(vertex_count() - 1);
                if (first.x != last.x || first.y != last.y) {
                    const V2 l[2] = {last, first};
                    curve(path, SPR_CURVE_LINEAR, l, 0.f);
                }
            }
            // the element's transform, applied to its vertices
            float m[6] = {1.f, 0.f, 0.f, 0.f, 1.f, 0.f};  // x' = m0 x + m1 y + m2, y' = m3 x + m4 y + m5
            if (t.compare(0, 10, "dyn_affine") == 0) {
                if (t.size() < 13) return SPR_ERR_INVALID_SCENE;
                std::string s = t.substr(12);
                for (const char *ch : {"]", "[", "]"}) {
                    const size_t k = s.find(ch);
                    if (k == std::string::npos) return SPR_ERR_INVALID_SCENE;
                    s.erase(k, 1);
                }
                if (s.empty()) return SPR_ERR_INVALID_SCENE;
                s = s.substr(0, s.length() - 1);
                separators_to_spaces(s);
                std::istringstream ms(s);
                ms >> m[0] >> m[1] >> m[2] >> m[3] >> m[4] >> m[5];
                for (uint32_t i = path_begin; i < vertex_count(); ++i) {
                    const float x = sc.vertex[2 * i], y = sc.vertex[2 * i + 1];
                    sc.vertex[2 * i] = (m[0] * x + m[1] * y) + m[2];
                    sc.vertex[2 * i + 1] = (m[3] * x + m[4] * y) + m[5];
                }
            } else if (t != "dyn_identity") {
                return SPR_ERR_INVALID_SCENE;
            }
            // paint
            float opacity = 1.f;
            if (!(in >> t) || t != "dyn_paint" || !(in >> opacity) || !(in >> t)) return SPR_ERR_INVALID_SCENE;
            if (t == "solid") {
                std::string c;
                if (!(in >> c)) return SPR_ERR_INVALID_SCENE;
                float r = 0.f, g = 0.f, b = 0.f, a = 1.f;
                if (c.compare(0, 4, "rgba") == 0 && c.size() >= 6) {
                    std::string v = c.substr(5, c.length() - 6);
                    separators_to_spaces(v);
                    std::istringstream vs(v);
                    vs >> r >> g >> b >> a;
                } else if (c.compare(0, 3, "rgb") == 0 && c.size() >= 6) {
                    std::string v = c.substr(4, c.length() - 6);
                    separators_to_spaces(v);
                    std::istringstream vs(v);
                    vs >> r >> g >> b;
                    a = 1.f;
                } else {
                    return SPR_ERR_INVALID_SCENE;
                }
                uint32_t ca = to_u8(a);
                const float sa = (float)ca * opacity;
                ca = sa > 0.f ? (sa >= 255.f ? 255u : (uint32_t)sa) : 0u;
                if (a128) {
                    ca = (uint32_t)(uint8_t)(((float)ca / 255.f) * 127.f);
                    ca = (uint32_t)(uint8_t)(((float)ca / 127.f) * 255.f);
                }
                const uint32_t rgba = to_u8(r) | (to_u8(g) << 8) | (to_u8(b) << 16) | (ca << 24);
                sc.fill_rgba[path] = (rgba & 0xFF000000u) ? rgba : 0u;
            } else if (t == "linear" || t == "radial") {
                skip_line();  // ramp stops and gradient transform
                sc.fill_rgba[path] = path + 1;
                ++info.n_gradient_paths;
            } else {
                return SPR_ERR_INVALID_SCENE;
            }
        }
        return SPR_OK;
    }
};

}  // namespace

extern "C" int spr_rvg_parse(const char *text, size_t length, int32_t a128, spr_scene **out, spr_rvg_info *info) {
    if (!text || !out) return SPR_ERR_INVALID_ARG;
    *out = nullptr;
    spr_scene *s = new (std::nothrow) spr_scene();
    if (!s) return SPR_ERR_OUT_OF_MEMORY;
    spr_rvg_info local{};
    Parser p(std::string(text, length), *s, local, a128 != 0);
    const int st = p.run();
    if (st) {
        delete s;
        return st;
    }
    if (info) *info = local;
    *out = s;
    return SPR_OK;
}

extern "C" int spr_rvg_load(const char *path, int32_t a128, spr_scene **out, spr_rvg_info *info) {
    if (!path || !out) return SPR_ERR_INVALID_ARG;
    std::ifstream f(path, std::ios::binary);
    if (!f) return SPR_ERR_INVALID_ARG;
    std::ostringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    return spr_rvg_parse(text.data(), text.size(), a128, out, info);
}
