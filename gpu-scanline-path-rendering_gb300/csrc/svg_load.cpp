// svg_load.cpp -- SVG documents into a host scene, following SVG::load
// (gpu-scanline/src/svg_load.cpp:189-1548) and the fill conversion of
// VGRasterizer::addVg (ras_base.cpp:142-166).
//
// What is read, as the reference reads it:
//   * the document's top-level <svg> elements: width, height, viewBox; the
//     output is the viewBox's size, vertices are moved by its origin and
//     flipped (y' = height - y) after loading (svg_load.cpp:1528-1545);
//   * <g> (presentation attributes, transform), <defs> (its children are
//     read like a group's, paths included), <path d>, <polygon points>,
//     <linearGradient>, <radialGradient>, <stop>; other elements are skipped
//     with their children;
//   * presentation attributes inherited down the tree: fill (none, a colour,
//     url(#id)), fill-rule, fill-opacity (multiplies the fill colour's
//     alpha), stroke (none, a colour, url(#id)), stroke-width, stroke-linecap
//     and stroke-linejoin (checked), transform; style with stop-color and
//     stop-opacity only;
//   * colours: rgb(r,g,b) (integers, truncated to 8 bits), #rgb, #rrggbb;
//   * transforms: matrix, translate (one value moves both axes by it),
//     scale; rotate, skewX and skewY are read and ignored (the reference
//     leaves them to a debug assert);
//   * path data M m L l H h V v C c S s Q q A a Z z with the reference's
//     reading: coordinates after the first pair of an M stay moves, Z closes
//     the contour with a line when its ends differ and keeps the current
//     point, S and T-less reflections use the last control point whatever
//     the previous command, arcs become cubics (addSVGArc,
//     vg_container.cpp:142-273, the endpoint-to-centre conversion of the SVG
//     implementation notes with one cubic per quarter turn, in the same mixed
//     float / double arithmetic);
//   * addVg's fill values: a colour with alpha 0 becomes 0; a stroked path is
//     filled, over its own geometry, with the stroke colour.
// Where the reference throws, hangs or reads uninitialised values, loading
// fails instead (the reference keeps the elements read before an exception):
// <rect> (the reference's reader table maps it to its line reader, which
// throws), <circle> and <ellipse> (read as rects with missing attributes),
// named colours and rgba(), a style key other than stop-color and
// stop-opacity, the color attribute (the reference pops the attribute stack
// on it), a T command or a character the path reader does not know after a
// number (the reference loops on it), a gradient referenced before it is
// defined, gradientUnits other than userSpaceOnUse.  Also defined here:
// a path element without d adds nothing (the reference re-styles the
// previous path); an arc with a zero radius is a line (the reference divides
// by zero); an arc that adds no curve leaves the current point; a document
// without viewBox takes (0, 0, width, height).
//
// Gradients: the reference's SVG loader records gradients but builds no
// gradient table (only its RVG loader does), so its gradient-filled SVG paths
// have no paint.  Here a linear or radial gradient fill gets the fill value
// path + 1 and a table item built as the RVG loader's (gradients.h), from the
// gradient's coordinates, stops (alpha times stop-opacity, as readStop
// does, then times fill-opacity), gradientTransform, the element's transform
// and the final flip; spread is pad.
//
// SPR_SVG_STROKE_TO_FILL: stroked paths keep their fill and get an outline
// path from spr_stroke_to_fill (width scaled by the square root of the
// element transform's determinant; gradient strokes get no outline) instead
// of addVg's stroke-colour fill.

#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/spr.h"
#include "gradients.h"
#include "spr_scene.h"

namespace {

// ---- a small XML reader: elements and attributes (entities decoded);
// text, comments, CDATA, processing instructions and DOCTYPE skipped ----

struct XNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<XNode> kids;
};

constexpr int kMaxDepth = 256;

struct XmlReader {
    const std::string &s;
    size_t i = 0;
    int depth = 0;
    explicit XmlReader(const std::string &text) : s(text) {}

    bool at(const char *t) const { return s.compare(i, std::strlen(t), t) == 0; }
    bool skip_past(const char *t) {
        const size_t k = s.find(t, i);
        if (k == std::string::npos) return false;
        i = k + std::strlen(t);
        return true;
    }
    void skip_ws() {
        while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
    }
    static bool name_char(char c) {
        const unsigned char u = (unsigned char)c;
        return std::isalnum(u) || c == '_' || c == ':' || c == '-' || c == '.' || u >= 0x80;
    }
    std::string name() {
        const size_t b = i;
        while (i < s.size() && name_char(s[i])) ++i;
        return s.substr(b, i - b);
    }
    static void utf8(uint32_t c, std::string &o) {
        if (c < 0x80) {
            o += (char)c;
        } else if (c < 0x800) {
            o += (char)(0xC0 | (c >> 6));
            o += (char)(0x80 | (c & 0x3F));
        } else if (c < 0x10000) {
            o += (char)(0xE0 | (c >> 12));
            o += (char)(0x80 | ((c >> 6) & 0x3F));
            o += (char)(0x80 | (c & 0x3F));
        } else {
            o += (char)(0xF0 | (c >> 18));
            o += (char)(0x80 | ((c >> 12) & 0x3F));
            o += (char)(0x80 | ((c >> 6) & 0x3F));
            o += (char)(0x80 | (c & 0x3F));
        }
    }
    // The five predefined entities and character references; anything else
    // stays as written.
    static std::string decode(const std::string &v) {
        std::string o;
        for (size_t k = 0; k < v.size();) {
            if (v[k] != '&') {
                o += v[k++];
                continue;
            }
            const size_t e = v.find(';', k);
            if (e == std::string::npos) {
                o += v[k++];
                continue;
            }
            const std::string ent = v.substr(k + 1, e - k - 1);
            static const std::map<std::string, char> named = {
                {"lt", '<'}, {"gt", '>'}, {"amp", '&'}, {"quot", '"'}, {"apos", '\''}};
            auto it = named.find(ent);
            if (it != named.end()) {
                o += it->second;
            } else if (ent.size() > 1 && ent[0] == '#') {
                const bool hex = ent[1] == 'x' || ent[1] == 'X';
                const std::string digits = ent.substr(hex ? 2 : 1);
                char *end = nullptr;
                const unsigned long c = std::strtoul(digits.c_str(), &end, hex ? 16 : 10);
                if (digits.empty() || *end || c == 0 || c > 0x10FFFF) {
                    o += v.substr(k, e - k + 1);
                } else {
                    utf8((uint32_t)c, o);
                }
            } else {
                o += v.substr(k, e - k + 1);
            }
            k = e + 1;
        }
        return o;
    }

    int element(XNode &n) {  // at '<' of a start tag
        ++i;
        n.name = name();
        if (n.name.empty()) return SPR_ERR_INVALID_SCENE;
        for (;;) {
            skip_ws();
            if (i >= s.size()) return SPR_ERR_INVALID_SCENE;
            if (at("/>")) {
                i += 2;
                return SPR_OK;
            }
            if (s[i] == '>') {
                ++i;
                if (++depth > kMaxDepth) return SPR_ERR_INVALID_SCENE;
                const int st = content(n.kids, &n.name);
                --depth;
                return st;
            }
            std::string an = name();
            if (an.empty()) return SPR_ERR_INVALID_SCENE;
            skip_ws();
            if (i >= s.size() || s[i] != '=') return SPR_ERR_INVALID_SCENE;
            ++i;
            skip_ws();
            if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) return SPR_ERR_INVALID_SCENE;
            const char q = s[i++];
            const size_t e = s.find(q, i);
            if (e == std::string::npos) return SPR_ERR_INVALID_SCENE;
            n.attrs.emplace_back(std::move(an), decode(s.substr(i, e - i)));
            i = e + 1;
        }
    }

    int content(std::vector<XNode> &kids, const std::string *close) {
        while (i < s.size()) {
            if (s[i] != '<') {
                ++i;
                continue;
            }
            if (at("<!--")) {
                if (!skip_past("-->")) return SPR_ERR_INVALID_SCENE;
            } else if (at("<![CDATA[")) {
                if (!skip_past("]]>")) return SPR_ERR_INVALID_SCENE;
            } else if (at("<?")) {
                if (!skip_past("?>")) return SPR_ERR_INVALID_SCENE;
            } else if (at("<!")) {
                int bracket = 0;
                for (i += 2; i < s.size(); ++i) {
                    if (s[i] == '[') ++bracket;
                    if (s[i] == ']') --bracket;
                    if (s[i] == '>' && bracket <= 0) break;
                }
                if (i >= s.size()) return SPR_ERR_INVALID_SCENE;
                ++i;
            } else if (at("</")) {
                i += 2;
                const std::string nm = name();
                skip_ws();
                if (i >= s.size() || s[i] != '>' || !close || nm != *close) return SPR_ERR_INVALID_SCENE;
                ++i;
                return SPR_OK;
            } else {
                kids.emplace_back();
                const int st = element(kids.back());
                if (st) return st;
            }
        }
        return close ? SPR_ERR_INVALID_SCENE : SPR_OK;
    }
};

// ---- numbers as sscanf("%f") / "%d" / "%x" read them ----

// Leading floats of s separated by white space (sscanf "%f %f ..."): the
// count read, at most n.
int scan_floats(const char *s, float *out, int n) {
    int k = 0;
    while (k < n) {
        char *end = nullptr;
        const float v = std::strtof(s, &end);
        if (end == s) break;
        out[k++] = v;
        s = end;
    }
    return k;
}

bool to_float(const std::string &s, float &v) { return scan_floats(s.c_str(), &v, 1) == 1; }

// "%d" then a literal ',' (no white space before it).
bool scan_int(const char *&p, int &v) {
    char *end = nullptr;
    const long x = std::strtol(p, &end, 10);
    if (end == p) return false;
    v = (int)x;
    p = end;
    return true;
}

bool hex_digits(const char *p, int w, int &v) {
    v = 0;
    for (int k = 0; k < w; ++k) {
        const int c = std::tolower((unsigned char)p[k]);
        if (c >= '0' && c <= '9') v = v * 16 + (c - '0');
        else if (c >= 'a' && c <= 'f') v = v * 16 + (c - 'a' + 10);
        else return false;
    }
    return true;
}

// ---- SVG state ----

struct V2 {
    float x, y;
};
bool operator!=(V2 a, V2 b) { return a.x != b.x || a.y != b.y; }

// glm::mat3 of an affine map: x' = a x + c y + e, y' = b x + d y + f.
struct Mat {
    float a = 1.f, b = 0.f, c = 0.f, d = 1.f, e = 0.f, f = 0.f;
};

// A * B with glm's column-major sums (the zero and one terms of the third
// row kept).
Mat mul(const Mat &A, const Mat &B) {
    Mat R;
    R.a = A.a * B.a + A.c * B.b + A.e * 0.f;
    R.b = A.b * B.a + A.d * B.b + A.f * 0.f;
    R.c = A.a * B.c + A.c * B.d + A.e * 0.f;
    R.d = A.b * B.c + A.d * B.d + A.f * 0.f;
    R.e = A.a * B.e + A.c * B.f + A.e * 1.f;
    R.f = A.b * B.e + A.d * B.f + A.f * 1.f;
    return R;
}

struct Rgba {
    uint8_t r = 0, g = 0, b = 0, a = 255;  // u8rgba() is opaque black
    uint32_t packed() const { return (uint32_t)r | ((uint32_t)g << 8) | ((uint32_t)b << 16) | ((uint32_t)a << 24); }
};

enum Paint { P_NONE, P_COLOR, P_GRADIENT };

struct Style {  // SVGPresentationAttribute
    Paint fill = P_COLOR;
    uint8_t rule = SPR_FILL_NONZERO;
    Rgba fill_color;
    int fill_index = -1;
    float fill_opacity = 1.f;
    Paint stroke = P_NONE;
    Rgba stroke_color;
    int stroke_index = -1;
    float stroke_width = 1.f;
    Mat m;
};

struct Stop {
    float offset = 0.f;
    Rgba color;
    float opacity = 1.f;
};

struct Gradient {
    bool radial = false;
    V2 v1{0.f, 0.f}, v2{0.f, 0.f}, c{0.f, 0.f}, f{0.f, 0.f};
    float r = 0.f;
    bool f_set = false;
    Mat m;
    std::vector<Stop> stops;
    std::string id;
};

struct PathRec {  // addPath's defaults until the element's style is applied: no fill
    Style style;
    PathRec() { style.fill = P_NONE; }
};

struct Loader {
    spr_scene &sc;
    spr_svg_info &info;
    bool a128;
    std::vector<Style> stack;
    std::vector<Gradient> gradients;
    std::map<std::string, int> gradient_ids;
    Gradient cur_gradient;
    Stop cur_stop;  // kept from stop to stop, as the reference's currentStop
    std::vector<PathRec> paths;
    float view_box[4] = {0.f, 0.f, 0.f, 0.f};
    bool have_view_box = false;
    float width_attr = 0.f, height_attr = 0.f;

    Loader(spr_scene &s, spr_svg_info &i, bool a) : sc(s), info(i), a128(a) {}

    Style &top() { return stack.back(); }
    uint32_t vertex_count() const { return (uint32_t)(sc.vertex.size() / 2); }
    V2 vertex(uint32_t k) const { return V2{sc.vertex[2 * k], sc.vertex[2 * k + 1]}; }

    void curve(uint32_t path, int type, const V2 *p, float w) {
        float xy[8];
        for (int k = 0; k < (type & 7); ++k) {
            xy[2 * k] = p[k].x;
            xy[2 * k + 1] = p[k].y;
        }
        sc.add_curve(path, type, xy, w);
    }

    int color(const std::string &str, Rgba &out) {  // parseColor
        const char *s = str.c_str();
        if (str.compare(0, 3, "rgb") == 0) {
            std::string t = str;
            for (size_t k = 4; k < t.size(); ++k)
                if (t[k] == ')') {
                    t[k] = ' ';
                    break;
                }
            if (t.size() < 4) return SPR_ERR_UNSUPPORTED;
            const char *p = t.c_str() + 4;
            int v[3];
            for (int k = 0; k < 3; ++k) {
                if (k && *p++ != ',') return SPR_ERR_UNSUPPORTED;
                if (!scan_int(p, v[k])) return SPR_ERR_UNSUPPORTED;  // rgba(...) lands here too
            }
            out = Rgba{(uint8_t)v[0], (uint8_t)v[1], (uint8_t)v[2], 255};
            return SPR_OK;
        }
        if (s[0] == '#') {
            int v[3];
            const int w = str.size() == 4 ? 1 : (str.size() == 7 ? 2 : 0);
            if (!w) return SPR_ERR_UNSUPPORTED;
            for (int k = 0; k < 3; ++k)
                if (!hex_digits(s + 1 + w * k, w, v[k])) return SPR_ERR_UNSUPPORTED;
            const int scale = w == 1 ? 17 : 1;
            out = Rgba{(uint8_t)(v[0] * scale), (uint8_t)(v[1] * scale), (uint8_t)(v[2] * scale), 255};
            return SPR_OK;
        }
        return SPR_ERR_UNSUPPORTED;  // named colours and the rest
    }

    int transform(const std::string &in, Mat &out) {  // parseTransform
        std::string t = in;
        for (char &ch : t)
            if (ch == ',' || ch == ' ' || ch == '\t' || ch == '\n' || ch == '\r') ch = ' ';
        Mat tm;
        size_t k = 0;
        for (;;) {
            while (k < t.size() && !std::isalpha((unsigned char)t[k])) ++k;
            if (k == t.size()) break;
            const size_t b = k;
            while (k < t.size() && std::isalpha((unsigned char)t[k])) ++k;
            if (k == t.size()) return SPR_ERR_INVALID_SCENE;
            const std::string label = t.substr(b, k - b);
            while (k < t.size() && t[k] != '(') ++k;
            if (k == t.size()) return SPR_ERR_INVALID_SCENE;
            const size_t vb = k + 1;
            while (k < t.size() && t[k] != ')') ++k;
            if (k == t.size()) return SPR_ERR_INVALID_SCENE;
            const std::string args = t.substr(vb, k - vb);
            ++k;
            float v[6];
            const int n = scan_floats(args.c_str(), v, 6);
            Mat m;
            if (label == "matrix") {
                if (n != 6) return SPR_ERR_INVALID_SCENE;
                m = Mat{v[0], v[1], v[2], v[3], v[4], v[5]};
            } else if (label == "translate") {
                if (n == 1) m.e = m.f = v[0];
                else if (n == 2) m.e = v[0], m.f = v[1];
                else return SPR_ERR_INVALID_SCENE;
            } else if (label == "scale") {
                if (n == 1) m.a = m.d = v[0];
                else if (n == 2) m.a = v[0], m.d = v[1];
                else return SPR_ERR_INVALID_SCENE;
            } else if (label != "rotate" && label != "skewX" && label != "skewY") {
                return SPR_ERR_INVALID_SCENE;
            }
            tm = mul(tm, m);
        }
        out = tm;
        return SPR_OK;
    }

    int paint_ref(const std::string &str, int &index) {  // url(#id)
        if (str.size() < 5) return SPR_ERR_INVALID_SCENE;
        std::string id = str.substr(4);
        id = id.substr(0, id.size() - 1);
        if (!id.empty() && id[0] == '#') id = id.substr(1);
        auto it = gradient_ids.find(id);
        if (it == gradient_ids.end()) return SPR_ERR_INVALID_SCENE;
        index = it->second;
        return SPR_OK;
    }

    // The default attribute reader: presentation attributes onto the top.
    int presentation(const std::string &k, const std::string &v, bool &used) {
        used = true;
        Style &s = top();
        if (k == "color") return SPR_ERR_UNSUPPORTED;
        if (k == "fill-rule") {
            if (v == "nonzero") s.rule = SPR_FILL_NONZERO;
            else if (v == "evenodd") s.rule = SPR_FILL_EVEN_ODD;
            return SPR_OK;
        }
        if (k == "fill-opacity") return to_float(v, s.fill_opacity) ? SPR_OK : SPR_ERR_INVALID_SCENE;
        if (k == "fill" || k == "stroke") {
            const bool fill = k == "fill";
            Paint &p = fill ? s.fill : s.stroke;
            if (v == "none") {
                p = P_NONE;
                return SPR_OK;
            }
            if (v.compare(0, 3, "url") == 0) {
                int gi;
                const int st = paint_ref(v, gi);
                if (st) return st;
                p = P_GRADIENT;
                (fill ? s.fill_index : s.stroke_index) = gi;
                return SPR_OK;
            }
            const int st = color(v, fill ? s.fill_color : s.stroke_color);
            if (st) return st;
            p = P_COLOR;
            return SPR_OK;
        }
        if (k == "stroke-width") return to_float(v, s.stroke_width) ? SPR_OK : SPR_ERR_INVALID_SCENE;
        if (k == "stroke-linecap")
            return v == "butt" || v == "round" || v == "square" ? SPR_OK : SPR_ERR_INVALID_SCENE;
        if (k == "stroke-linejoin")
            return v == "miter" || v == "round" || v == "bevel" ? SPR_OK : SPR_ERR_INVALID_SCENE;
        if (k == "transform") {
            Mat m;
            const int st = transform(v, m);
            if (st) return st;
            s.m = mul(s.m, m);
            return SPR_OK;
        }
        if (k == "style") {
            size_t b = 0;
            while (b < v.size()) {
                size_t e = v.find(';', b);
                if (e == std::string::npos) e = v.size();
                const std::string item = v.substr(b, e - b);
                b = e + 1;
                const size_t colon = item.find(':');
                if (colon == std::string::npos) return SPR_ERR_INVALID_SCENE;
                const std::string key = item.substr(0, colon), val = item.substr(colon + 1);
                if (key == "stop-color") {
                    const int st = color(val, cur_stop.color);
                    if (st) return st;
                } else if (key == "stop-opacity") {
                    if (!to_float(val, cur_stop.opacity)) return SPR_ERR_INVALID_SCENE;
                } else {
                    return SPR_ERR_UNSUPPORTED;
                }
            }
            return SPR_OK;
        }
        // read and without effect here
        if (k == "opacity" || k == "stroke-opacity" || k == "stroke-miterlimit" || k == "stroke-dasharray" ||
            k == "stroke-dashoffset" || k == "visibility")
            return SPR_OK;
        used = false;
        return SPR_OK;
    }

    // ar_path_d: one path of contours from path data.
    int path_data(const std::string &d) {
        if (d.empty()) return SPR_OK;
        const uint32_t path = (uint32_t)paths.size();
        paths.push_back(PathRec{});
        uint32_t contour_first = vertex_count(), contour_curves = 0;
        enum { CMD, NUMBER } state = CMD;
        char cmd = 0;
        bool rel = false;
        char num[256];
        int num_len = 0;
        float value[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        int vi = 0;
        V2 lp0{0.f, 0.f}, lp1{0.f, 0.f};  // current point, last control point
        auto pt = [&](const float *a) {
            V2 p{a[0], a[1]};
            if (rel) p = V2{p.x + lp0.x, p.y + lp0.y};
            return p;
        };
        auto add = [&](int type, const V2 *p, float w) {
            curve(path, type, p, w);
            ++contour_curves;
        };
        const size_t n = d.size();
        for (size_t i = 0; i <= n;) {
            const char cc = i == n ? '\0' : d[i];
            if (state == CMD) {
                rel = std::islower((unsigned char)cc) != 0;
                const char lc = (char)std::tolower((unsigned char)cc);
                switch (lc) {
                case 'm':
                    if (contour_curves) {
                        contour_first = vertex_count();
                        contour_curves = 0;
                    }
                    cmd = lc;
                    state = NUMBER;
                    break;
                case 'l': case 'h': case 'v': case 'q': case 'c': case 's': case 'a':
                    cmd = lc;
                    state = NUMBER;
                    break;
                case 'z': {
                    if (contour_first == vertex_count()) break;
                    const V2 fv = vertex(contour_first), lv = vertex(vertex_count() - 1);
                    if (fv != lv) {
                        const V2 l[2] = {lv, fv};
                        add(SPR_CURVE_LINEAR, l, 0.f);
                    }
                    break;
                }
                default:  // white space and unknown characters (T among them) are passed over
                    break;
                }
                ++i;
                continue;
            }
            const bool digitish = std::isdigit((unsigned char)cc) || cc == 'e' || cc == 'E' || cc == '.';
            const bool minus = cc == '-' && (num_len == 0 || std::tolower((unsigned char)num[num_len - 1]) == 'e');
            if (digitish || minus) {
                if (num_len >= 255) return SPR_ERR_INVALID_SCENE;
                num[num_len++] = cc;
                ++i;
                continue;
            }
            if (num_len) {  // a number ends
                num[num_len] = '\0';
                num_len = 0;
                char *end = nullptr;
                const float v = std::strtof(num, &end);
                if (end == num) return SPR_ERR_INVALID_SCENE;
                value[vi++] = v;
                V2 p[4];
                switch (cmd) {
                case 'm':
                    if (vi == 2) {
                        lp0 = pt(value);
                        vi = 0;
                    }
                    break;
                case 'l':
                    if (vi == 2) {
                        p[0] = lp0;
                        p[1] = pt(value);
                        add(SPR_CURVE_LINEAR, p, 0.f);
                        lp0 = p[1];
                        vi = 0;
                    }
                    break;
                case 'h':
                    p[0] = lp0;
                    p[1] = V2{rel ? lp0.x + value[0] : value[0], lp0.y};
                    add(SPR_CURVE_LINEAR, p, 0.f);
                    lp0 = p[1];
                    vi = 0;
                    break;
                case 'v':
                    p[0] = lp0;
                    p[1] = V2{lp0.x, rel ? lp0.y + value[0] : value[0]};
                    add(SPR_CURVE_LINEAR, p, 0.f);
                    lp0 = p[1];
                    vi = 0;
                    break;
                case 'c':
                    if (vi == 6) {
                        p[0] = lp0;
                        p[1] = pt(value);
                        p[2] = pt(value + 2);
                        p[3] = pt(value + 4);
                        add(SPR_CURVE_CUBIC, p, 0.f);
                        lp0 = p[3];
                        lp1 = p[2];
                        vi = 0;
                    }
                    break;
                case 's':
                    if (vi == 4) {
                        p[0] = lp0;
                        p[1] = V2{lp0.x + (lp0.x - lp1.x), lp0.y + (lp0.y - lp1.y)};
                        p[2] = pt(value);
                        p[3] = pt(value + 2);
                        add(SPR_CURVE_CUBIC, p, 0.f);
                        lp0 = p[3];
                        lp1 = p[2];
                        vi = 0;
                    }
                    break;
                case 'q':
                    if (vi == 4) {
                        p[0] = lp0;
                        p[1] = pt(value);
                        p[2] = pt(value + 2);
                        add(SPR_CURVE_QUADRATIC, p, 0.f);
                        lp0 = p[2];
                        lp1 = p[1];
                        vi = 0;
                    }
                    break;
                case 'a':
                    if (vi == 7) {
                        const uint32_t before = vertex_count();
                        arc(path, lp0, value[0], value[1], value[2], (int)value[3], (int)value[4], pt(value + 5),
                            contour_curves);
                        if (vertex_count() != before) {
                            lp0 = vertex(vertex_count() - 1);
                            lp1 = vertex(vertex_count() - 2);
                        }
                        vi = 0;
                    }
                    break;
                default:
                    return SPR_ERR_INVALID_SCENE;
                }
            }
            switch (std::tolower((unsigned char)cc)) {
            case ' ': case '\t': case '\n': case '\r': case ',': case '\0':
                ++i;
                break;
            case 'm': case 'l': case 'h': case 'v': case 'q': case 'c': case 's': case 'a': case 'z':
                state = CMD;
                break;
            case '-':
                break;
            default:  // the reference's reader never advances past this character
                return SPR_ERR_UNSUPPORTED;
            }
        }
        return SPR_OK;
    }

    // addSVGArc: endpoint to centre parameterisation, then one cubic per
    // quarter turn or less with handle length 8/3 sin^2(d/4) / sin(d/2) of
    // the radius.
    void arc(uint32_t path, V2 start, float rx_in, float ry_in, float rot, int large, int sweep, V2 end,
             uint32_t &contour_curves) {
        if (rx_in == 0.f || ry_in == 0.f) {
            const V2 l[2] = {start, end};
            curve(path, SPR_CURVE_LINEAR, l, 0.f);
            ++contour_curves;
            return;
        }
        const double kPi = std::acos(-1.0);
        const double kRad = std::acos(-1.0) / 180.0;
        auto vector_angle = [&](double ux, double uy, double vx, double vy) {
            const double ta = std::atan2(uy, ux), tb = std::atan2(vy, vx);
            return tb >= ta ? tb - ta : kPi * 2 - (ta - tb);
        };
        const double sin_phi = std::sin(rot * kRad), cos_phi = std::cos(rot * kRad);
        const double x1d = cos_phi * (start.x - end.x) / 2.0 + sin_phi * (start.y - end.y) / 2.0;
        const double y1d = -sin_phi * (start.x - end.x) / 2.0 + cos_phi * (start.y - end.y) / 2.0;
        const float rr = rx_in * rx_in * ry_in * ry_in;  // float products, as the reference's
        const double numerator = rr - rx_in * rx_in * y1d * y1d - ry_in * ry_in * x1d * x1d;
        float rx = rx_in, ry = ry_in;
        double root;
        if (numerator < 0.0) {
            const float s = (float)std::sqrt(1.0 - numerator / rr);
            rx *= s;
            ry *= s;
            root = 0.0;
        } else {
            const bool neg = (large == 1 && sweep == 1) || (large == 0 && sweep == 0);
            root = (neg ? -1.0 : 1.0) * std::sqrt(numerator / (rx_in * rx_in * y1d * y1d + ry_in * ry_in * x1d * x1d));
        }
        const double cxd = root * rx * y1d / ry, cyd = -root * ry * x1d / rx;
        const double cx = cos_phi * cxd - sin_phi * cyd + (start.x + end.x) / 2.0;
        const double cy = sin_phi * cxd + cos_phi * cyd + (start.y + end.y) / 2.0;
        double theta1 = vector_angle(1.0, 0.0, (x1d - cxd) / rx, (y1d - cyd) / ry);
        double dtheta = vector_angle((x1d - cxd) / rx, (y1d - cyd) / ry, (-x1d - cxd) / rx, (-y1d - cyd) / ry);
        if (sweep == 0 && dtheta > 0) dtheta -= 2.0 * kPi;
        else if (sweep == 1 && dtheta < 0) dtheta += 2.0 * kPi;
        const int segments = (int)std::ceil(std::fabs(dtheta / (kPi / 2.0)));
        const double delta = dtheta / segments;
        const double t = 8.0 / 3.0 * std::sin(delta / 4.0) * std::sin(delta / 4.0) / std::sin(delta / 2.0);
        double sx = start.x, sy = start.y;
        for (int k = 0; k < segments; ++k) {
            const double c1 = std::cos(theta1), s1 = std::sin(theta1);
            const double theta2 = theta1 + delta;
            const double c2 = std::cos(theta2), s2 = std::sin(theta2);
            const double ex = cos_phi * rx * c2 - sin_phi * ry * s2 + cx;
            const double ey = sin_phi * rx * c2 + cos_phi * ry * s2 + cy;
            const double dx1 = t * (-cos_phi * rx * s1 - sin_phi * ry * c1);
            const double dy1 = t * (-sin_phi * rx * s1 + cos_phi * ry * c1);
            const double dxe = t * (cos_phi * rx * s2 + sin_phi * ry * c2);
            const double dye = t * (sin_phi * rx * s2 - cos_phi * ry * c2);
            const V2 p[4] = {V2{(float)sx, (float)sy}, V2{(float)(sx + dx1), (float)(sy + dy1)},
                             V2{(float)(ex + dxe), (float)(ey + dye)}, V2{(float)ex, (float)ey}};
            curve(path, SPR_CURVE_CUBIC, p, 0.f);
            ++contour_curves;
            theta1 = theta2;
            sx = (float)ex;
            sy = (float)ey;
        }
    }

    // Applies the top style to the last path and transforms its vertices
    // (readPath / readPolygon).
    void finish_path(uint32_t vbegin) {
        Style &a = top();
        a.fill_color.a = (uint8_t)((float)a.fill_color.a * a.fill_opacity);
        if (a128) {
            a.fill_color.a = (uint8_t)(((float)a.fill_color.a / 255.f) * 127.f);
            a.fill_color.a = (uint8_t)(((float)a.fill_color.a / 127.f) * 255.f);
        }
        paths.back().style = a;
        const Mat &m = a.m;
        for (uint32_t k = vbegin; k < vertex_count(); ++k) {
            const float x = sc.vertex[2 * k], y = sc.vertex[2 * k + 1];
            sc.vertex[2 * k] = m.a * x + m.c * y + m.e * 1.f;
            sc.vertex[2 * k + 1] = m.b * x + m.d * y + m.f * 1.f;
        }
    }

    int read_path(const XNode &n) {
        const uint32_t vbegin = vertex_count();
        const size_t paths_before = paths.size();
        for (const auto &kv : n.attrs) {
            bool used;
            int st = presentation(kv.first, kv.second, used);
            if (st) return st;
            if (!used && kv.first == "d") {
                st = path_data(kv.second);
                if (st) return st;
            }
        }
        if (paths.size() == paths_before) return SPR_OK;  // no path data: nothing to style
        finish_path(vbegin);
        return SPR_OK;
    }

    int read_polygon(const XNode &n) {
        const uint32_t vbegin = vertex_count();
        for (const auto &kv : n.attrs) {
            bool used;
            int st = presentation(kv.first, kv.second, used);
            if (st) return st;
            if (!used && kv.first == "d") {
                st = path_data(kv.second);
                if (st) return st;
            }
        }
        const uint32_t path = (uint32_t)paths.size();
        paths.push_back(PathRec{});
        for (const auto &kv : n.attrs) {
            if (kv.first != "points") continue;
            std::string v = kv.second;
            for (char &ch : v)
                if (ch == ',') ch = ' ';
            std::istringstream in(v);
            in.imbue(std::locale::classic());
            V2 vf{0.f, 0.f}, v0, v1;
            in >> vf.x >> vf.y;
            v0 = vf;
            while (in >> v1.x >> v1.y) {
                const V2 l[2] = {v0, v1};
                curve(path, SPR_CURVE_LINEAR, l, 0.f);
                v0 = v1;
            }
            const V2 l[2] = {v0, vf};
            curve(path, SPR_CURVE_LINEAR, l, 0.f);
        }
        finish_path(vbegin);
        return SPR_OK;
    }

    int read_gradient(const XNode &n, bool radial) {
        stack.push_back(top());
        cur_gradient = Gradient{};
        cur_gradient.radial = radial;
        for (const auto &kv : n.attrs) {
            const std::string &k = kv.first, &v = kv.second;
            float x = 0.f;
            int st = SPR_OK;
            if (k == "id") {
                cur_gradient.id = v;
            } else if (k == "gradientTransform") {
                st = transform(v, cur_gradient.m);
            } else if (k == "gradientUnits") {
                if (v != "userSpaceOnUse") st = SPR_ERR_UNSUPPORTED;
            } else if (k == "spreadMethod") {
            } else if ((!radial && (k == "x1" || k == "y1" || k == "x2" || k == "y2")) ||
                       (radial && (k == "cx" || k == "cy" || k == "r" || k == "fx" || k == "fy"))) {
                if (!to_float(v, x)) return SPR_ERR_INVALID_SCENE;
                Gradient &g = cur_gradient;
                if (k == "x1") g.v1.x = x;
                else if (k == "y1") g.v1.y = x;
                else if (k == "x2") g.v2.x = x;
                else if (k == "y2") g.v2.y = x;
                else if (k == "cx") g.c.x = x;
                else if (k == "cy") g.c.y = x;
                else if (k == "r") g.r = x;
                else if (k == "fx") g.f.x = x, g.f_set = true;
                else g.f.y = x, g.f_set = true;
            } else {
                bool used;
                st = presentation(k, v, used);
            }
            if (st) return st;
        }
        const int st = children(n);
        if (st) return st;
        if (radial && !cur_gradient.f_set) cur_gradient.f = cur_gradient.c;
        gradients.push_back(cur_gradient);
        gradient_ids[cur_gradient.id] = (int)gradients.size() - 1;
        stack.pop_back();
        return SPR_OK;
    }

    int read_stop(const XNode &n) {
        stack.push_back(top());
        for (const auto &kv : n.attrs) {
            const std::string &k = kv.first, &v = kv.second;
            int st = SPR_OK;
            if (k == "offset") {
                if (!to_float(v, cur_stop.offset)) return SPR_ERR_INVALID_SCENE;
            } else if (k == "stop-color") {
                st = color(v, cur_stop.color);
            } else if (k == "stop-opacity") {
                if (!to_float(v, cur_stop.opacity)) return SPR_ERR_INVALID_SCENE;
            } else {
                bool used;
                st = presentation(k, v, used);
            }
            if (st) return st;
        }
        cur_stop.color.a = (uint8_t)((float)cur_stop.color.a * cur_stop.opacity);
        cur_gradient.stops.push_back(cur_stop);
        stack.pop_back();
        return SPR_OK;
    }

    int element(const XNode &n) {  // readDefault's dispatch
        const std::string &nm = n.name;
        int st = SPR_OK;
        if (nm == "defs") {
            st = children(n);
        } else if (nm == "g") {
            stack.push_back(top());
            for (const auto &kv : n.attrs) {
                bool used;
                st = presentation(kv.first, kv.second, used);
                if (st) return st;
            }
            st = children(n);
            stack.pop_back();
        } else if (nm == "path") {
            stack.push_back(top());
            st = read_path(n);
            stack.pop_back();
        } else if (nm == "polygon") {
            stack.push_back(top());
            st = read_polygon(n);
            stack.pop_back();
        } else if (nm == "rect" || nm == "circle" || nm == "ellipse") {
            st = SPR_ERR_UNSUPPORTED;
        } else if (nm == "linearGradient" || nm == "radialGradient") {
            st = read_gradient(n, nm == "radialGradient");
        } else if (nm == "stop") {
            st = read_stop(n);
        }
        return st;
    }

    int children(const XNode &n) {
        for (const XNode &k : n.kids) {
            const int st = element(k);
            if (st) return st;
        }
        return SPR_OK;
    }

    int svg(const XNode &n) {
        for (const auto &kv : n.attrs) {
            if (kv.first == "width" || kv.first == "height") {
                float v;
                if (!to_float(kv.second, v)) return SPR_ERR_INVALID_SCENE;
                (kv.first == "width" ? width_attr : height_attr) = v;
            } else if (kv.first == "viewBox") {
                std::string t = kv.second;
                float v[4];
                if (scan_floats(t.c_str(), v, 4) != 4) return SPR_ERR_INVALID_SCENE;
                std::memcpy(view_box, v, sizeof(v));
                have_view_box = true;
            }
        }
        stack.push_back(Style{});
        const int st = children(n);
        stack.pop_back();
        return st;
    }
};

int load(const std::string &text, int32_t flags, spr_scene **out, spr_svg_info *info_out) {
    std::vector<XNode> top;
    XmlReader xr(text);
    int st = xr.content(top, nullptr);
    if (st) return st;
    spr_scene *s = new (std::nothrow) spr_scene();
    if (!s) return SPR_ERR_OUT_OF_MEMORY;
    spr_svg_info info{};
    Loader ld(*s, info, (flags & SPR_SVG_A128) != 0);
    try {
        for (const XNode &n : top)
            if (n.name == "svg" && (st = ld.svg(n)) != SPR_OK) break;
    } catch (const std::bad_alloc &) {
        st = SPR_ERR_OUT_OF_MEMORY;
    }
    if (!st && !ld.have_view_box) {
        ld.view_box[0] = ld.view_box[1] = 0.f;
        ld.view_box[2] = ld.width_attr;
        ld.view_box[3] = ld.height_attr;
    }
    const int W = (int)ld.view_box[2], H = (int)ld.view_box[3];
    if (!st && (W <= 0 || H <= 0)) st = SPR_ERR_INVALID_SCENE;
    if (st) {
        delete s;
        return st;
    }
    // the viewBox origin and the flip to y up
    for (size_t k = 0; k < s->vertex.size(); k += 2) {
        s->vertex[k] -= ld.view_box[0];
        const float y = s->vertex[k + 1] - ld.view_box[1];
        s->vertex[k + 1] = (float)H - y;
    }
    // addVg's paths, fill values and gradient items
    const bool srgb = (flags & SPR_SVG_SRGB_RAMPS) != 0, outline = (flags & SPR_SVG_STROKE_TO_FILL) != 0;
    Mat flip;
    flip.d = -1.f;
    flip.e = -ld.view_box[0];
    flip.f = (float)H + ld.view_box[1];
    spr_grad::Builder grads;
    std::vector<spr_stroke_style> styles;
    bool any_gradient = false;
    for (size_t p = 0; p < ld.paths.size(); ++p) {
        const Style &a = ld.paths[p].style;
        uint32_t fill = 0;
        s->fill_rule.push_back(a.rule);
        if (a.fill == P_COLOR) {
            const uint32_t c = a.fill_color.packed();
            fill = (c & 0xFF000000u) ? c : 0u;
        }
        if (a.fill == P_GRADIENT) {
            const Gradient &g = ld.gradients[(size_t)a.fill_index];
            const Mat m = mul(flip, mul(a.m, g.m));
            const float tr[6] = {m.a, m.c, m.e, m.b, m.d, m.f};
            std::vector<float> k;
            for (const Stop &stp : g.stops)
                k.insert(k.end(), {stp.offset, stp.color.r / 255.f, stp.color.g / 255.f, stp.color.b / 255.f,
                                   stp.color.a / 255.f * a.fill_opacity});
            if (g.radial) grads.paint(true, tr, g.c.x, g.c.y, g.f.x, g.f.y, g.r, k, srgb);
            else grads.paint(false, tr, g.v1.x, g.v1.y, g.v2.x, g.v2.y, 0.f, k, srgb);
            fill = (uint32_t)p + 1;
            any_gradient = true;
            ++info.n_gradient_paths;
        } else {
            grads.solid();
        }
        spr_stroke_style ss{0u, 0.f};
        if (a.stroke == P_COLOR) {
            const uint32_t c = a.stroke_color.packed();
            ++info.n_stroked_paths;
            if (outline) {
                ss.rgba = (c & 0xFF000000u) ? c : 0u;
                ss.width = a.stroke_width * std::sqrt(std::fabs(a.m.a * a.m.d - a.m.b * a.m.c));
            } else {
                fill = (c & 0xFF000000u) ? c : 0u;
            }
        }
        s->fill_rgba.push_back(fill);
        styles.push_back(ss);
    }
    if (any_gradient) grads.finish(*s);
    if (outline && !s->fill_rule.empty()) {
        spr_scene_view v;
        spr_scene_view_of(s, &v);
        spr_scene *o = nullptr;
        st = spr_stroke_to_fill(&v, styles.data(), &o, nullptr);
        if (st) {
            delete s;
            return st;
        }
        o->grad_table = std::move(s->grad_table);
        o->grad_ramp = std::move(s->grad_ramp);
        delete s;
        s = o;
    }
    info.view_box[0] = ld.view_box[0];
    info.view_box[1] = ld.view_box[1];
    info.view_box[2] = ld.view_box[2];
    info.view_box[3] = ld.view_box[3];
    info.width = W;
    info.height = H;
    info.n_paths = (int32_t)s->fill_rule.size();
    if (info_out) *info_out = info;
    *out = s;
    return SPR_OK;
}

}  // namespace

extern "C" int spr_svg_parse(const char *text, size_t length, int32_t flags, spr_scene **out, spr_svg_info *info) {
    if (!out || (!text && length)) return SPR_ERR_INVALID_ARG;
    *out = nullptr;
    try {
        return load(std::string(text ? text : "", length), flags, out, info);
    } catch (const std::bad_alloc &) {
        return SPR_ERR_OUT_OF_MEMORY;
    }
}

extern "C" int spr_svg_load(const char *path, int32_t flags, spr_scene **out, spr_svg_info *info) {
    if (!out || !path) return SPR_ERR_INVALID_ARG;
    *out = nullptr;
    std::ifstream f(path, std::ios::binary);
    if (!f) return SPR_ERR_INVALID_ARG;
    std::ostringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    return spr_svg_parse(text.data(), text.size(), flags, out, info);
}
