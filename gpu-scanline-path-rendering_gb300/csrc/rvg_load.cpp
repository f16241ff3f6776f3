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
// become 0.  Linear and radial paints get the fill value path + 1 and an
// entry in the gradient table (12 words per painted path: the inverse
// gradient transform, ramp position and length, focal point) with their
// colour ramp sampled into the ramp texels, as the reference builds
// gradient_table_texture and gradient_ramp_texture (rvg.cpp:487-760).  The
// reference's parsing quirks are kept: rgb() drops the last character of its
// third number, the three points after dyn_concrete are read and ignored.

#include <algorithm>
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
#include "gradients.h"
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

// f32tou8 of rvg.cpp: truncation, clamped to 0..255
uint32_t f32tou8(float a) {
    int r = (int)(a * 255.f);
    if (r > 255) r = 255;
    if (r < 0) r = 0;
    return (uint32_t)r;
}

float safe_rcp(float a) { return a != 0.f ? 1.f / a : 0.f; }

float srgb_to_linear(float f) { return f <= 0.04045f ? f / 12.92f : std::pow((f + 0.055f) / (1.f + 0.055f), 2.4f); }

float linear_to_srgb(float f) { return f <= 0.0031308f ? 12.92f * f : (1.f + 0.055f) * std::pow(f, 1.f / 2.4f) - 0.055f; }

}  // namespace

namespace spr_grad {

// The paint's gradient item and ramp (rvg.cpp:487-700): the inverse of the
// paint-to-scene map followed by the gradient's own normalisation, the
// focal point, and the stops sampled into 2^k texels (16 per smallest stop
// gap, at most 1024).
void Builder::paint(bool radial, const float tr[6], float x0, float y0, float x1, float y1, float r,
                    std::vector<float> k, bool srgb) {
    float ti[6] = {1.f, 0.f, 0.f, 0.f, 1.f, 0.f};
    float focal[3] = {0.f, 0.f, 0.f};
    const float det = (float)((double)tr[0] * (double)tr[4] - (double)tr[1] * (double)tr[3]);
    const float idet = safe_rcp(det);
    ti[0] = tr[4] * idet;
    ti[3] = -tr[3] * idet;
    ti[1] = -tr[1] * idet;
    ti[4] = tr[0] * idet;
    ti[2] = -(float)((double)tr[2] * (double)ti[0] + (double)tr[5] * (double)ti[1]);
    ti[5] = -(float)((double)tr[2] * (double)ti[3] + (double)tr[5] * (double)ti[4]);
    ti[2] -= x0;
    ti[5] -= y0;
    if (radial) {
        const float ir = safe_rcp(r);
        for (float &v : ti) v *= ir;
        focal[0] = (x1 - x0) * ir;
        focal[1] = (y1 - y0) * ir;
    } else {
        float dx = x1 - x0, dy = y1 - y0;
        const float kk = 2.f / (dx * dx + dy * dy);
        dx *= kk;
        dy *= kk;
        ti[0] = ti[0] * dx + ti[3] * dy;
        ti[1] = ti[1] * dx + ti[4] * dy;
        ti[2] = ti[2] * dx + ti[5] * dy;
        ti[3] = ti[4] = ti[5] = 0.f;
        ti[2] -= 1.f;
        focal[0] = -1.f;
        focal[1] = 0.f;
    }
    focal[2] = 1.f - focal[0] * focal[0] - focal[1] * focal[1];
    if (!(focal[2] > 0.f)) focal[2] = 0.f;
    if (k.empty()) k.assign(5, 0.f);
    if (k.size() <= 5) {
        k.resize(10);
        std::memcpy(&k[5], &k[0], sizeof(float) * 5);
        k[0] = 0.f;
        k[5] = 1.f;
    }
    float min_delta = 1.f;
    for (size_t i = 5; i < k.size(); i += 5) {
        const float d = k[i] - k[i - 5];
        if (d > 0.f && d < min_delta) min_delta = d;
    }
    int res = (int)(16.f / min_delta);
    if (res < 1) res = 1;
    if (res > 1023) res = 1023;
    res |= res >> 1;
    res |= res >> 2;
    res |= res >> 4;
    res |= res >> 8;
    res++;
    Item gi{};
    std::memcpy(gi.tr, ti, sizeof(ti));
    std::memcpy(gi.focal, focal, sizeof(focal));
    gi.mode = radial ? 1 : 0;
    gi.p = (int32_t)ramp.size();
    gi.n = res;
    items.push_back(gi);
    const float ires = 1.f / (float)(res - 1);
    size_t pk = 0;
    for (int i = 0; i < res; ++i) {
        const float t = (float)i * ires;
        float t0 = 0.f, t1 = 1.f;
        while (pk + 10 < k.size()) {
            t0 = k[pk];
            t1 = k[pk + 5];
            if (t > t1 || t0 == t1) pk += 5;
            else break;
        }
        t0 = k[pk];
        t1 = k[pk + 5];
        float tl = (t - t0) * safe_rcp(t1 - t0);
        if (!(tl > 0.f)) tl = 0.f;
        if (tl > 1.f) tl = 1.f;
        auto lerp = [](float a, float b, float u) { return a + (b - a) * u; };
        uint32_t rgba;
        if (srgb) {  // interpolated in linear light, stored as sRGB
            auto mix = [](float a, float b, float u) { return a * (1 - u) + b * u; };
            float c[3];
            for (int ch = 0; ch < 3; ++ch)
                c[ch] = linear_to_srgb(mix(srgb_to_linear(k[pk + 1 + ch]), srgb_to_linear(k[pk + 6 + ch]), tl));
            rgba = f32tou8(c[0]) | (f32tou8(c[1]) << 8) | (f32tou8(c[2]) << 16);
        } else {
            rgba = f32tou8(lerp(k[pk + 1], k[pk + 6], tl)) | (f32tou8(lerp(k[pk + 2], k[pk + 7], tl)) << 8) |
                   (f32tou8(lerp(k[pk + 3], k[pk + 8], tl)) << 16);
        }
        rgba += f32tou8(lerp(k[pk + 4], k[pk + 9], tl)) << 24;
        ramp.push_back(rgba);
    }
}

// gradient_table_texture / gradient_ramp_texture: ramps repacked by
// decreasing length (a ramp of 2^k texels then never crosses a 1024-texel
// row), 12 words per painted path, (n - 1) / 1024 in word 7.
void Builder::finish(spr_scene &sc) {
    const size_t n = items.size();
    std::vector<size_t> order(n);
    for (size_t i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return items[a].n > items[b].n; });
    sc.grad_ramp.assign((ramp.size() + 1023) / 1024 * 1024, 0u);
    int32_t pout = 0;
    for (size_t id : order) {
        const int32_t p0 = items[id].p;
        items[id].p = pout;
        if (items[id].n) {
            std::memcpy(&sc.grad_ramp[pout], &ramp[p0], sizeof(uint32_t) * items[id].n);
            pout += items[id].n;
        }
    }
    sc.grad_table.assign(std::max<size_t>(n, 1) * 12, 0u);
    for (size_t i = 0; i < n; ++i) {
        std::memcpy(&sc.grad_table[i * 12], &items[i], 12 * sizeof(uint32_t));
        const float scale = (float)(items[i].n - 1) * (1.f / 1024.f);
        std::memcpy(&sc.grad_table[i * 12 + 7], &scale, 4);
    }
}

}  // namespace spr_grad

namespace {

struct Parser {
    std::istringstream in;
    spr_scene &sc;
    spr_rvg_info &info;
    bool a128, srgb;
    spr_grad::Builder grads;  // one item per painted path
    Parser(const std::string &text, spr_scene &s, spr_rvg_info &i, bool a, bool sr)
        : in(text), sc(s), info(i), a128(a), srgb(sr) {}

    // The rest of a linear / radial paint line: stops, then "pad", then the
    // gradient transform (rvg.cpp:487-700).
    int gradient(bool radial, float opacity) {
        std::string line;
        std::getline(in, line);
        const size_t ppad = line.find("pad");
        if (ppad == std::string::npos) return SPR_ERR_INVALID_SCENE;
        const size_t n = line.size();
        for (size_t i = 0; i < n; ++i) {
            const int ch = (int)(uint8_t)line[i];
            if ((uint32_t)(ch - 48) >= 10u && ch != '-' && ch != '.' && ch != '+' &&
                !(ch == 'e' && i + 1 < n && (line[i + 1] == '+' || line[i + 1] == '-')))
                line[i] = ' ';
        }
        std::istringstream s0(line.substr(0, ppad)), s1(line.substr(ppad));
        float tr[6] = {1.f, 0.f, 0.f, 0.f, 1.f, 0.f};
        s1 >> tr[0] >> tr[1] >> tr[2] >> tr[3] >> tr[4] >> tr[5];
        float x0 = 0.f, y0 = 0.f, x1 = 0.f, y1 = 0.f, r = 0.f;
        s0 >> x0 >> y0 >> x1 >> y1;
        if (radial) s0 >> r;
        // stops: offset and RGBA (alpha times the opacity)
        std::vector<float> k;
        float knot = 0.f;
        while (s0 >> knot) {
            float v[4] = {0.f, 0.f, 0.f, 0.f};
            s0 >> v[0] >> v[1] >> v[2] >> v[3];
            k.insert(k.end(), {knot, v[0], v[1], v[2], v[3] * opacity});
        }
        grads.paint(radial, tr, x0, y0, x1, y1, r, k, srgb);
        return SPR_OK;
    }

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
                grads.solid();  // an empty slot keeps the table indexed by path
            } else if (t == "linear" || t == "radial") {
                const int st = gradient(t == "radial", opacity);
                if (st) return st;
                sc.fill_rgba[path] = path + 1;
                ++info.n_gradient_paths;
            } else {
                return SPR_ERR_INVALID_SCENE;
            }
        }
        grads.finish(sc);
        return SPR_OK;
    }
};

}  // namespace

extern "C" int spr_rvg_parse(const char *text, size_t length, int32_t flags, spr_scene **out, spr_rvg_info *info) {
    if (!text || !out) return SPR_ERR_INVALID_ARG;
    *out = nullptr;
    spr_scene *s = new (std::nothrow) spr_scene();
    if (!s) return SPR_ERR_OUT_OF_MEMORY;
    spr_rvg_info local{};
    int st;
    try {  // no C++ exception crosses the C ABI: an allocation failure is a status
        Parser p(std::string(text, length), *s, local, (flags & SPR_RVG_A128) != 0,
                 (flags & SPR_RVG_SRGB_RAMPS) != 0);
        st = p.run();
    } catch (const std::bad_alloc &) {
        st = SPR_ERR_OUT_OF_MEMORY;
    }
    if (st) {
        delete s;
        return st;
    }
    if (info) *info = local;
    *out = s;
    return SPR_OK;
}

extern "C" int spr_rvg_load(const char *path, int32_t flags, spr_scene **out, spr_rvg_info *info) {
    if (!path || !out) return SPR_ERR_INVALID_ARG;
    *out = nullptr;
    try {
        std::ifstream f(path, std::ios::binary);
        if (!f) return SPR_ERR_INVALID_ARG;
        std::ostringstream ss;
        ss << f.rdbuf();
        const std::string text = ss.str();
        return spr_rvg_parse(text.data(), text.size(), flags, out, info);
    } catch (const std::bad_alloc &) {
        return SPR_ERR_OUT_OF_MEMORY;
    }
}

extern "C" int spr_scene_gradients(const spr_scene *s, const uint32_t **table, uint32_t *n_entries,
                                   const uint32_t **ramp, uint32_t *n_texels) {
    if (!s || !table || !n_entries || !ramp || !n_texels) return SPR_ERR_INVALID_ARG;
    *table = s->grad_table.empty() ? nullptr : s->grad_table.data();
    *n_entries = (uint32_t)(s->grad_table.size() / 12);
    *ramp = s->grad_ramp.empty() ? nullptr : s->grad_ramp.data();
    *n_texels = (uint32_t)s->grad_ramp.size();
    return SPR_OK;
}
