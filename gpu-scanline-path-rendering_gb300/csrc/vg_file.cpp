// vg_file.cpp -- the reference's own scene files: VGContainer::saveBinary /
// loadBinary (.vgb) and saveTxt / loadTxt (.vgt), vg_container.cpp:1667-1911,
// read into a host scene with the flattening of VGRasterizer::addVg
// (ras_base.cpp:138-230): paths in order, each path's contours in order, each
// contour's curves in order; fill value = colour (0 if its alpha is 0) for
// colour fills, path + 1 for gradient fills, 0 otherwise.
//
// Both formats hold: x, y, width, height; the counts of paths, contours,
// curves, vertices, ramp texels and gradient-table words; per path its first
// contour, contour count, fill type (1 colour, 4 gradient), fill rule, RGBA8
// colour and gradient index; per contour its first curve and curve count; per
// curve its first vertex, type and the rational weight's float bits; the
// vertices; the ramp texels; the gradient table.  .vgb stores them as arrays
// in that order (little-endian); .vgt one record per line, comma-separated,
// with the type and rule bytes written as raw characters.

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

constexpr uint8_t kFillColor = 1, kFillGradient = 4;

struct Container {
    int32_t x = 0, y = 0, width = 0, height = 0;
    std::vector<uint32_t> contour_index, contour_number, fill_color, fill_index;
    std::vector<uint8_t> fill_type, fill_rule;
    std::vector<uint32_t> curve_index, curve_number;   // per contour
    std::vector<uint32_t> vertex_index, arc_w;        // per curve
    std::vector<uint8_t> type;                        // per curve
    std::vector<float> vertex;                        // x, y
    std::vector<uint32_t> ramp, table;
};

bool ends_with(const std::string &s, const char *suffix) {
    const size_t n = std::strlen(suffix);
    return s.size() >= n && s.compare(s.size() - n, n, suffix) == 0;
}

// ---- .vgb ------------------------------------------------------------------
struct Reader {
    const std::string &b;
    size_t pos = 0;
    bool ok = true;
    template <class T>
    void get(std::vector<T> &v, size_t n) {
        v.resize(n);
        if (pos + n * sizeof(T) > b.size()) {
            ok = false;
            return;
        }
        if (n) std::memcpy(v.data(), b.data() + pos, n * sizeof(T));
        pos += n * sizeof(T);
    }
    uint32_t u32() {
        std::vector<uint32_t> v;
        get(v, 1);
        return ok ? v[0] : 0u;
    }
};

int read_vgb(const std::string &bytes, Container &c) {
    Reader r{bytes};
    c.x = (int32_t)r.u32();
    c.y = (int32_t)r.u32();
    c.width = (int32_t)r.u32();
    c.height = (int32_t)r.u32();
    const uint32_t np = r.u32(), nc = r.u32(), ncu = r.u32(), nv = r.u32(), nr = r.u32(), nt = r.u32();
    if (!r.ok) return SPR_ERR_INVALID_SCENE;
    // every count must fit the file before anything is allocated
    const uint64_t need = 40ull + 14ull * np + 8ull * nc + 9ull * ncu + 8ull * nv + 4ull * nr + 4ull * nt;
    if (need > bytes.size()) return SPR_ERR_INVALID_SCENE;
    r.get(c.contour_index, np);
    r.get(c.contour_number, np);
    r.get(c.fill_type, np);
    r.get(c.fill_rule, np);
    r.get(c.fill_color, np);
    r.get(c.fill_index, np);
    r.get(c.curve_index, nc);
    r.get(c.curve_number, nc);
    r.get(c.vertex_index, ncu);
    r.get(c.type, ncu);
    r.get(c.arc_w, ncu);
    r.get(c.vertex, 2 * (size_t)nv);
    r.get(c.ramp, nr);
    r.get(c.table, nt);
    return r.ok ? SPR_OK : SPR_ERR_INVALID_SCENE;
}

template <class T>
void put(std::string &out, const std::vector<T> &v) {
    out.append(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(T));
}

void put_u32(std::string &out, uint32_t v) { out.append(reinterpret_cast<const char *>(&v), 4); }

std::string write_vgb(const Container &c) {
    std::string out;
    for (int32_t v : {c.x, c.y, c.width, c.height}) put_u32(out, (uint32_t)v);
    for (size_t v : {c.fill_type.size(), c.curve_index.size(), c.type.size(), c.vertex.size() / 2, c.ramp.size(),
                     c.table.size()})
        put_u32(out, (uint32_t)v);
    put(out, c.contour_index);
    put(out, c.contour_number);
    put(out, c.fill_type);
    put(out, c.fill_rule);
    put(out, c.fill_color);
    put(out, c.fill_index);
    put(out, c.curve_index);
    put(out, c.curve_number);
    put(out, c.vertex_index);
    put(out, c.type);
    put(out, c.arc_w);
    put(out, c.vertex);
    put(out, c.ramp);
    put(out, c.table);
    return out;
}

// ---- .vgt ------------------------------------------------------------------
// A cursor over the text with the scanf conversions the reference's loadTxt
// uses (%d, %u, %e, %c, literal ',', whitespace before numbers).
struct Text {
    const std::string &s;
    size_t pos = 0;
    bool ok = true;
    void skip_space() {
        while (pos < s.size() && (s[pos] == ' ' || s[pos] == '\n' || s[pos] == '\r' || s[pos] == '\t')) ++pos;
    }
    void lit(char ch) {
        if (pos < s.size() && s[pos] == ch) ++pos;
        else ok = false;
    }
    long long integer() {
        skip_space();
        size_t used = 0;
        long long v = 0;
        try {
            v = std::stoll(s.substr(pos, 24), &used);
        } catch (...) {
            ok = false;
            return 0;
        }
        pos += used;
        return v;
    }
    float real() {
        skip_space();
        size_t used = 0;
        float v = 0.f;
        try {
            v = std::stof(s.substr(pos, 48), &used);
        } catch (...) {
            ok = false;
            return 0.f;
        }
        pos += used;
        return v;
    }
    uint8_t byte() {  // %c: any character, no skipping
        if (pos >= s.size()) {
            ok = false;
            return 0;
        }
        return (uint8_t)s[pos++];
    }
};

int read_vgt(const std::string &text, Container &c) {
    Text t{text};
    c.x = (int32_t)t.integer();
    t.lit(',');
    c.y = (int32_t)t.integer();
    t.lit(',');
    c.width = (int32_t)t.integer();
    t.lit(',');
    c.height = (int32_t)t.integer();
    uint32_t n[6];
    for (int i = 0; i < 6; ++i) {
        if (i) t.lit(',');
        n[i] = (uint32_t)t.integer();
    }
    if (!t.ok) return SPR_ERR_INVALID_SCENE;
    // each record takes at least two characters
    const uint64_t records = (uint64_t)n[0] + n[1] + n[2] + n[3] + n[4] + n[5];
    if (2 * records > text.size()) return SPR_ERR_INVALID_SCENE;
    const uint32_t np = n[0], nc = n[1], ncu = n[2], nv = n[3], nr = n[4], nt = n[5];
    c.contour_index.resize(np);
    c.contour_number.resize(np);
    c.fill_type.resize(np);
    c.fill_rule.resize(np);
    c.fill_color.resize(np);
    c.fill_index.resize(np);
    for (uint32_t i = 0; i < np && t.ok; ++i) {
        c.contour_index[i] = (uint32_t)t.integer();
        t.lit(',');
        c.contour_number[i] = (uint32_t)t.integer();
        t.lit(',');
        c.fill_type[i] = t.byte();
        t.lit(',');
        c.fill_rule[i] = t.byte();
        t.lit(',');
        c.fill_color[i] = (uint32_t)t.integer();
        t.lit(',');
        c.fill_index[i] = (uint32_t)t.integer();
    }
    c.curve_index.resize(nc);
    c.curve_number.resize(nc);
    for (uint32_t i = 0; i < nc && t.ok; ++i) {
        c.curve_index[i] = (uint32_t)t.integer();
        t.lit(',');
        c.curve_number[i] = (uint32_t)t.integer();
    }
    c.vertex_index.resize(ncu);
    c.type.resize(ncu);
    c.arc_w.resize(ncu);
    for (uint32_t i = 0; i < ncu && t.ok; ++i) {
        c.vertex_index[i] = (uint32_t)t.integer();
        t.lit(',');
        c.type[i] = t.byte();
        t.lit(',');
        c.arc_w[i] = (uint32_t)(int32_t)t.integer();
    }
    c.vertex.resize(2 * (size_t)nv);
    for (uint32_t i = 0; i < nv && t.ok; ++i) {
        c.vertex[2 * i] = t.real();
        t.lit(',');
        c.vertex[2 * i + 1] = t.real();
    }
    c.ramp.resize(nr);
    for (uint32_t i = 0; i < nr && t.ok; ++i) c.ramp[i] = (uint32_t)(int32_t)t.integer();
    c.table.resize(nt);
    for (uint32_t i = 0; i < nt && t.ok; ++i) c.table[i] = (uint32_t)(int32_t)t.integer();
    return t.ok ? SPR_OK : SPR_ERR_INVALID_SCENE;
}

std::string write_vgt(const Container &c) {
    std::string out;
    char line[160];
    std::snprintf(line, sizeof(line), "%d,%d,%d,%d\n", c.x, c.y, c.width, c.height);
    out += line;
    std::snprintf(line, sizeof(line), "%u,%u,%u,%u,%u,%u\n", (unsigned)c.fill_type.size(),
                  (unsigned)c.curve_index.size(), (unsigned)c.type.size(), (unsigned)(c.vertex.size() / 2),
                  (unsigned)c.ramp.size(), (unsigned)c.table.size());
    out += line;
    for (size_t i = 0; i < c.fill_type.size(); ++i) {
        std::snprintf(line, sizeof(line), "%u,%u,", c.contour_index[i], c.contour_number[i]);
        out += line;
        out += (char)c.fill_type[i];
        out += ',';
        out += (char)c.fill_rule[i];
        std::snprintf(line, sizeof(line), ",%u,%u\n", c.fill_color[i], c.fill_index[i]);
        out += line;
    }
    for (size_t i = 0; i < c.curve_index.size(); ++i) {
        std::snprintf(line, sizeof(line), "%u,%u\n", c.curve_index[i], c.curve_number[i]);
        out += line;
    }
    for (size_t i = 0; i < c.type.size(); ++i) {
        std::snprintf(line, sizeof(line), "%u,", c.vertex_index[i]);
        out += line;
        out += (char)c.type[i];
        std::snprintf(line, sizeof(line), ",%d\n", (int32_t)c.arc_w[i]);
        out += line;
    }
    for (size_t i = 0; i < c.vertex.size() / 2; ++i) {
        std::snprintf(line, sizeof(line), "%e,%e\n", (double)c.vertex[2 * i], (double)c.vertex[2 * i + 1]);
        out += line;
    }
    for (uint32_t v : c.ramp) {
        std::snprintf(line, sizeof(line), "%d\n", (int32_t)v);
        out += line;
    }
    for (uint32_t v : c.table) {
        std::snprintf(line, sizeof(line), "%d\n", (int32_t)v);
        out += line;
    }
    return out;
}

// ---- container <-> scene ------------------------------------------------------
// addVg's flattening (ras_base.cpp:138-230).
int to_scene(const Container &c, spr_scene &s) {
    const uint32_t np = (uint32_t)c.fill_type.size(), nc = (uint32_t)c.curve_index.size();
    const uint32_t ncu = (uint32_t)c.type.size(), nv = (uint32_t)(c.vertex.size() / 2);
    s.vertex = c.vertex;
    for (uint32_t p = 0; p < np; ++p) {
        uint32_t fill = 0u;
        if (c.fill_type[p] == kFillColor) fill = (c.fill_color[p] & 0xFF000000u) ? c.fill_color[p] : 0u;
        else if (c.fill_type[p] == kFillGradient) fill = p + 1;
        s.fill_rgba.push_back(fill);
        s.fill_rule.push_back(c.fill_rule[p] ? SPR_FILL_EVEN_ODD : SPR_FILL_NONZERO);
        for (uint32_t k = 0; k < c.contour_number[p]; ++k) {
            const uint64_t con = (uint64_t)c.contour_index[p] + k;
            if (con >= nc) return SPR_ERR_INVALID_SCENE;
            for (uint32_t j = 0; j < c.curve_number[con]; ++j) {
                const uint64_t cu = (uint64_t)c.curve_index[con] + j;
                if (cu >= ncu) return SPR_ERR_INVALID_SCENE;
                const int type = c.type[cu];
                if (type != SPR_CURVE_LINEAR && type != SPR_CURVE_QUADRATIC && type != SPR_CURVE_CUBIC &&
                    type != SPR_CURVE_RATIONAL)
                    return SPR_ERR_INVALID_SCENE;
                if ((uint64_t)c.vertex_index[cu] + (type & 7) > nv) return SPR_ERR_INVALID_SCENE;
                // every curve owns its vertices, so the curves of all paths together
                // name at most nv of them: stop before paths that share contours
                // make the arrays grow past the file's own size
                if (s.vertex_path_id.size() + (size_t)(type & 7) > nv) return SPR_ERR_INVALID_SCENE;
                s.curve_vertex_pos.push_back(c.vertex_index[cu]);
                s.curve_type.push_back((uint8_t)type);
                s.curve_path_id.push_back(p);
                float w = -1.f;
                if (type == SPR_CURVE_RATIONAL) std::memcpy(&w, &c.arc_w[cu], 4);
                s.curve_arc_w.push_back(w);
                for (int v = 0; v < (type & 7); ++v) s.vertex_path_id.push_back(p);
            }
        }
    }
    // addVg numbers the vertices' paths curve by curve (the vertex array's own
    // order when each curve owns its vertices in turn); the counts must agree
    if (s.vertex_path_id.size() != nv) return SPR_ERR_INVALID_SCENE;
    s.grad_ramp = c.ramp;
    s.grad_table = c.table;
    return SPR_OK;
}

// One contour per path holding the path's curves in order.
void from_scene(const spr_scene &s, int32_t width, int32_t height, Container &c) {
    c.width = width;
    c.height = height;
    const uint32_t np = (uint32_t)s.fill_rule.size(), ncu = (uint32_t)s.curve_type.size();
    std::vector<uint32_t> first(np, 0u), count(np, 0u);
    for (uint32_t i = 0; i < ncu; ++i) {
        const uint32_t p = s.curve_path_id[i];
        if (count[p] == 0) first[p] = i;
        ++count[p];
    }
    for (uint32_t p = 0; p < np; ++p) {
        c.contour_index.push_back(p);
        c.contour_number.push_back(1u);
        const uint32_t f = s.fill_rgba[p];
        const bool grad = s.grad_table.size() >= 12 && f >= 1u && f - 1u < 0x01000000u;
        c.fill_type.push_back(grad ? kFillGradient : kFillColor);
        c.fill_rule.push_back(s.fill_rule[p]);
        c.fill_color.push_back(grad ? 0x00FF00FFu : f);
        c.fill_index.push_back(grad ? p : 0xFFFFFFFFu);
        c.curve_index.push_back(first[p]);
        c.curve_number.push_back(count[p]);
    }
    for (uint32_t i = 0; i < ncu; ++i) {
        c.vertex_index.push_back(s.curve_vertex_pos[i]);
        c.type.push_back(s.curve_type[i]);
        uint32_t w = 0u;
        if (s.curve_type[i] == SPR_CURVE_RATIONAL) std::memcpy(&w, &s.curve_arc_w[i], 4);
        c.arc_w.push_back(w);
    }
    c.vertex = s.vertex;
    c.ramp = s.grad_ramp;
    c.table = s.grad_table;
}

}  // namespace

namespace {
int vg_load(const char *path, spr_scene **out, spr_vg_info *info) {
    const std::string name(path);
    const bool bin = ends_with(name, "vgb"), txt = ends_with(name, "vgt");
    if (!bin && !txt) return SPR_ERR_INVALID_ARG;
    std::ifstream f(path, std::ios::binary);
    if (!f) return SPR_ERR_INVALID_ARG;
    std::ostringstream ss;
    ss << f.rdbuf();
    const std::string bytes = ss.str();
    Container c;
    int st = bin ? read_vgb(bytes, c) : read_vgt(bytes, c);
    if (st) return st;
    spr_scene *s = new (std::nothrow) spr_scene();
    if (!s) return SPR_ERR_OUT_OF_MEMORY;
    if ((st = to_scene(c, *s))) {
        delete s;
        return st;
    }
    if (info) {
        info->x = c.x;
        info->y = c.y;
        info->width = c.width;
        info->height = c.height;
        info->n_contours = (int32_t)c.curve_index.size();
    }
    *out = s;
    return SPR_OK;
}

int vg_save(const spr_scene *s, int32_t width, int32_t height, const char *path) {
    const std::string name(path);
    const bool bin = ends_with(name, "vgb"), txt = ends_with(name, "vgt");
    if (!bin && !txt) return SPR_ERR_INVALID_ARG;
    if (s->has_affine) return SPR_ERR_UNSUPPORTED;  // the format has no per-path transforms
    Container c;
    from_scene(*s, width, height, c);
    const std::string bytes = bin ? write_vgb(c) : write_vgt(c);
    std::ofstream f(path, std::ios::binary);
    if (!f) return SPR_ERR_INVALID_ARG;
    f.write(bytes.data(), (std::streamsize)bytes.size());
    return f ? SPR_OK : SPR_ERR_INVALID_ARG;
}

int scene_from_view(const spr_scene_view *v, spr_scene *s) {
    s->vertex.assign(v->vertex, v->vertex + 2 * (size_t)v->n_vertices);
    s->vertex_path_id.assign(v->vertex_path_id, v->vertex_path_id + v->n_vertices);
    s->curve_vertex_pos.assign(v->curve_vertex_pos, v->curve_vertex_pos + v->n_curves);
    s->curve_type.assign(v->curve_type, v->curve_type + v->n_curves);
    s->curve_path_id.assign(v->curve_path_id, v->curve_path_id + v->n_curves);
    s->curve_arc_w.assign(v->n_curves, -1.f);
    if (v->curve_arc_w) s->curve_arc_w.assign(v->curve_arc_w, v->curve_arc_w + v->n_curves);
    s->fill_rule.assign(v->path_fill_rule, v->path_fill_rule + v->n_paths);
    s->fill_rgba.assign(v->path_fill_rgba, v->path_fill_rgba + v->n_paths);
    if (v->path_affine) {
        s->affine.assign(v->path_affine, v->path_affine + 6 * (size_t)v->n_paths);
        s->has_affine = true;
    }
    return SPR_OK;
}
}  // namespace

// The C entry points: no C++ exception crosses the ABI (an allocation failure
// on a large or hostile file is a status, not std::terminate).
extern "C" int spr_vg_load(const char *path, spr_scene **out, spr_vg_info *info) {
    if (!path || !out) return SPR_ERR_INVALID_ARG;
    *out = nullptr;
    try {
        return vg_load(path, out, info);
    } catch (const std::bad_alloc &) {
        return SPR_ERR_OUT_OF_MEMORY;
    }
}

extern "C" int spr_vg_save(const spr_scene *s, int32_t width, int32_t height, const char *path) {
    if (!s || !path) return SPR_ERR_INVALID_ARG;
    try {
        return vg_save(s, width, height, path);
    } catch (const std::bad_alloc &) {
        return SPR_ERR_OUT_OF_MEMORY;
    }
}

extern "C" int spr_scene_from_view(const spr_scene_view *v, spr_scene **out) {
    if (!v || !out) return SPR_ERR_INVALID_ARG;
    *out = nullptr;
    const int st = spr_validate_scene(v);
    if (st) return st;
    spr_scene *s = new (std::nothrow) spr_scene();
    if (!s) return SPR_ERR_OUT_OF_MEMORY;
    int r;
    try {
        r = scene_from_view(v, s);
    } catch (const std::bad_alloc &) {
        r = SPR_ERR_OUT_OF_MEMORY;
    }
    if (r) {
        delete s;
        return r;
    }
    *out = s;
    return SPR_OK;
}

extern "C" int spr_scene_set_gradients(spr_scene *s, const uint32_t *table, uint32_t n_entries,
                                       const uint32_t *ramp, uint32_t n_texels) {
    if (!s || (n_entries && !table) || (n_texels && !ramp)) return SPR_ERR_INVALID_ARG;
    s->grad_table.assign(table, table + 12 * (size_t)n_entries);
    s->grad_ramp.assign(ramp, ramp + n_texels);
    return SPR_OK;
}
