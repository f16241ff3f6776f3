// spr_oracle.cpp -- CPU restatement of the reference's comb-scanline fill
// pipeline, stage by stage.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA product
// path is compared against; it is compiled into liboracle (never into libspr)
// and only tests/, __graft_entry__.smoke() and bench.py's CPU legs load it.
//
// Every stage cites the reference function it restates ("cu" below is
// gpu-scanline/src/rasterizer/R_cut_A_mask_comb_scanline/ras_cut_mask_comb_scanline.cu,
// "ras_cut.h" and friends live in gpu-scanline/src/rasterizer/shared/).
//
// Floating point: compiled with -ffp-contract=off so that every a*b+c is two
// rounded operations, exactly as the CUDA kernels compiled with --fmad=false.
// Conversions and shifts follow the CUDA/PTX semantics the reference relies
// on (saturating float->int, NaN->0, shift counts >= width give 0); see the
// helpers below.

#include "spr_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------- helpers --
struct F2 {
    float x, y;
};

inline uint32_t bits_of(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
inline float float_of(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// __float2int_rd: floor, saturating, NaN -> 0.
inline int32_t cvt_rmi(float x) {
    if (std::isnan(x)) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x < -2147483648.0f) return INT32_MIN;
    return (int32_t)std::floor(x);
}
// (int)float: truncation, saturating, NaN -> 0 (cvt.rzi.s32.f32).
inline int32_t cvt_rzi(float x) {
    if (std::isnan(x)) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x < -2147483648.0f) return INT32_MIN;
    return (int32_t)x;
}
// (int)double: truncation, saturating, NaN -> 0 (cvt.rzi.s32.f64).
inline int32_t cvt_rzi_d(double x) {
    if (std::isnan(x)) return 0;
    if (x >= 2147483648.0) return INT32_MAX;
    if (x <= -2147483649.0) return INT32_MIN;
    return (int32_t)x;
}
// 32-bit wrapping subtraction a - b.
inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
// Logical shifts with counts outside [0, width) giving 0 (PTX clamps the
// count to the register width).
inline uint32_t shr32(uint32_t v, int32_t s) { return (s < 0 || s >= 32) ? 0u : (v >> s); }
inline uint64_t shr64(uint64_t v, int32_t s) { return (s < 0 || s >= 64) ? 0ull : (v >> s); }

// fmaxf/fminf: NaN operands are ignored, +0 wins over -0 for max and -0 over
// +0 for min.
inline float fmax_r(float a, float b) {
    if (std::isnan(a)) return b;
    if (std::isnan(b)) return a;
    if (a > b) return a;
    if (b > a) return b;
    return std::signbit(a) ? b : a;
}
inline float fmin_r(float a, float b) {
    if (std::isnan(a)) return b;
    if (std::isnan(b)) return a;
    if (a < b) return a;
    if (b < a) return b;
    return std::signbit(a) ? a : b;
}

// cutil_math.h:862-864 and 1019-1022.
inline float safe_rcp(float a) { return a != 0.f ? (1.f / a) : 0.f; }
inline float lerp(float a, float b, float t) { return a + t * (b - a); }

constexpr int kLinear = SPR_CURVE_LINEAR;
constexpr int kQuad = SPR_CURVE_QUADRATIC;
constexpr int kCubic = SPR_CURVE_CUBIC;
constexpr int kRational = SPR_CURVE_RATIONAL;

// One coordinate of a curve point: interpolateGeneralCurve (ras_cut.h:586-632)
// and d_curve_point / bezier_curve_point (bezier_curve.h:58-150); for a
// rational curve `v[1]` is the raw middle coordinate, multiplied by w here.
inline float curve_coord(int type, float w, const float *v, float t) {
    switch (type) {
    case kLinear:
        return lerp(v[0], v[1], t);
    case kQuad: {
        float a = lerp(v[0], v[1], t);
        float b = lerp(v[1], v[2], t);
        return lerp(a, b, t);
    }
    case kCubic: {
        float q0 = lerp(v[0], v[1], t);
        float q1 = lerp(v[1], v[2], t);
        float q2 = lerp(v[2], v[3], t);
        float l0 = lerp(q0, q1, t);
        float l1 = lerp(q1, q2, t);
        return lerp(l0, l1, t);
    }
    default: {  // rational quadratic
        float iv1 = v[1] * w;
        float l0 = lerp(v[0], iv1, t);
        float l1 = lerp(iv1, v[2], t);
        float r = lerp(l0, l1, t);
        float ww = (1 - t) * (1 - t) + 2.f * (1 - t) * t * w + t * t;
        r *= safe_rcp(ww);
        return r;
    }
    }
}

// solveQuadEquation (ras_cut.h:33-64).
inline void solve_quad_eq(float a, float b, float c, float *r0, float *r1) {
    if (a == 0) {
        float x = -c / b;
        *r0 = x;
        *r1 = x;
        return;
    }
    float A = a;
    float B = (float)((double)b * 0.5);
    float C = c;
    float tx, ty;
    float R = B * B - A * C;
    if (R > 0.0f) {
        float SR = std::sqrt(R);
        if (B > 0.0f) {
            float TB = B + SR;
            tx = -C / TB;
            ty = -TB / A;
        } else {
            float TB = -B + SR;
            tx = TB / A;
            ty = C / TB;
        }
    } else {
        tx = 0.f;
        ty = 0.f;
    }
    *r0 = tx;
    *r1 = ty;
}

// solveQuadBezierQM (ras_cut.h:373-388).
inline float solve_quad_bezier(float iA, float iB, float iC, float iD, float t0, float t1) {
    float a = iA + (-2.f) * iB + iC;
    float b = -2.f * iA + 2.f * iB;
    float c = iA - iD;
    float r0 = 0.f, r1 = 0.f;
    solve_quad_eq(a, b, c, &r0, &r1);
    if (t0 <= r0 && r0 <= t1) return r0;
    if (t0 <= r1 && r1 <= t1) return r1;
    return t0;
}

inline int32_t floor2(float x) { return (int32_t)((uint32_t)cvt_rmi(x) & 0xFFFFFFFEu); }

// ------------------------------------------------------------- parallel --
void parallel_for(int threads, int64_t n, const std::function<void(int64_t, int64_t)> &fn) {
    if (n <= 0) return;
    int t = threads;
    if (t <= 1 || n < 4096) {
        fn(0, n);
        return;
    }
    int64_t chunks = std::min<int64_t>(n, (int64_t)t * 8);
    std::atomic<int64_t> next{0};
    std::vector<std::thread> pool;
    for (int i = 0; i < t; ++i) {
        pool.emplace_back([&]() {
            for (;;) {
                int64_t c = next.fetch_add(1);
                if (c >= chunks) break;
                int64_t b = n * c / chunks, e = n * (c + 1) / chunks;
                fn(b, e);
            }
        });
    }
    for (auto &th : pool) th.join();
}

// --------------------------------------------------------------- tables --
// Sample positions of one pixel: vg_sample_position (ras_qm_mask.cu:118-175).
// 32 samples: rows y = (2i+1)/64, columns x = (k_i + 0.5)/96.  8 samples: row
// i of 8, column = bit-reversed i (own bit length) scaled to 8 columns.
const uint8_t kCol32[32] = {0, 50, 24, 74, 12, 62, 38, 84, 6,  54, 30, 80, 18, 68, 42, 92,
                            3, 53, 29, 77, 17, 63, 41, 89, 9,  59, 35, 83, 21, 71, 45, 93};

std::vector<F2> pixel_samples(int n) {
    std::vector<F2> s(n);
    if (n == 32) {
        for (int i = 0; i < 32; ++i) {
            s[i].x = (float)((kCol32[i] + 0.5) / 96.0);
            s[i].y = (float)((2 * i + 1) / 64.0);
        }
    } else {
        // 8 samples: ras_qm_mask.cu:130-163; 16 samples (an extension, no
        // counterpart in the reference) apply the same rule to 16 rows.
        const double gap = 1.0 / n, hgap = gap / 2;
        for (int i = 0; i < n; ++i) {
            int x = i, y = 0, bc = 0;
            while (x) {
                y = (y << 1) | (x & 1);
                x >>= 1;
                ++bc;
            }
            double f = y / (float)(1 << bc);
            int col = (int)(f * n);
            s[i].x = (float)(col * gap + hgap);
            s[i].y = (float)(i * gap + hgap);
        }
        // sort_samples (ras_qm_mask.cu:44-48): by y, then x.  Already ordered.
        std::stable_sort(s.begin(), s.end(), [](const F2 &a, const F2 &b) {
            return (a.y < b.y) || (a.y == b.y && a.x < b.x);
        });
    }
    return s;
}

// 256 samples (an extension) apply the 8-sample rule to 256 rows and are
// rendered as 8 passes of 32: pass g holds rows 8j + g (j < 32), each moved
// to the 32-sample row (2j + 1) / 64, and the pass moves the geometry up by
// (2g - 7) / 512 pixel instead (row 8j + g sits at (16j + 2g + 1) / 512).
std::vector<F2> pass_samples_256(int g) {
    std::vector<F2> all = pixel_samples(256), s(32);
    for (int j = 0; j < 32; ++j) s[j] = F2{all[8 * j + g].x, (float)((2 * j + 1) / 64.0)};
    return s;
}

inline float pass_shift_256(int g) { return (float)(2 * g - 7) / 512.f; }

// Samples of the 2x2 cell (init_qm_mask_table, ras_qm_mask.h:734-759).
std::vector<F2> cell_samples_of(const std::vector<F2> &p) {
    const int n = (int)p.size();
    std::vector<F2> c(4 * n);
    const float ox[4] = {0, 0, 1, 1}, oy[4] = {0, 1, 0, 1};
    for (int k = 0; k < 4; ++k)
        for (int i = 0; i < n; ++i) {
            F2 v{p[i].x + ox[k], p[i].y + oy[k]};
            c[k * n + i] = F2{v.x * .5f, v.y * .5f};
        }
    return c;
}

std::vector<F2> cell_samples(int n) { return cell_samples_of(pixel_samples(n)); }

inline F2 normalize2(F2 v) {
    float inv = 1.0f / std::sqrt(v.x * v.x + v.y * v.y);
    return F2{v.x * inv, v.y * inv};
}

// QM_Mask_2x2::makeTable (ras_qm_mask.h:432-484), built on the host.  Words
// per texel: samples/8 (8 spp: one word, 32 spp: four).
std::vector<uint32_t> mask_table_of(const std::vector<F2> &cs) {
    const int n = (int)cs.size() / 4;
    const int words = n / 8;
    std::vector<uint32_t> t((size_t)65536 * words);
    for (int i = 0; i < 65536; ++i) {
        int y = i / 256, x = i - y * 256;
        float xf = ((float)x + 0.5f) * (1.f / 256.f);
        float yf = ((float)y + 0.5f) * (1.f / 256.f);
        F2 nr{2.f * (xf - 0.5f), 2.f * (yf - 0.5f)};
        float lg2 = nr.x * nr.x + nr.y * nr.y;
        float lg = std::sqrt(lg2);
        float inv = 1.f / lg;
        F2 N{inv * nr.x, inv * nr.y};
        float C = fmax_r(1.f - lg, 0.f) * (1.f / 0.5f);
        if (N.x < 0.f) {
            N = F2{-N.x, -N.y};
            C = -C;
        }
        if (x == 37 && y == 218) {
            N = normalize2(F2{1.f, -1.f});
            C = 0.f;
        }
        C += 0.5f * (N.x + N.y);
        for (int w = 0; w < words; ++w) {
            uint32_t m = 0;
            for (int j = 0; j < 32; ++j) {
                F2 P = cs[w * 32 + j];
                if (N.x * P.x + N.y * P.y - C > 0.f) m |= 1u << j;
            }
            t[(size_t)i * words + w] = m;
        }
    }
    return t;
}

std::vector<uint32_t> build_mask_table(int n) { return mask_table_of(cell_samples(n)); }

std::vector<uint32_t> build_pass_mask_table_256(int g) { return mask_table_of(cell_samples_of(pass_samples_256(g))); }

// fetchPixelTable (ras_qm_mask.h:519-542) with the texture replaced by an
// explicit point-sampled, clamped lookup: texel = clamp(floor(uv * 256)).
inline void fetch_pixel_table(const uint32_t *table, int words, F2 P0, F2 P1, uint32_t *out) {
    if (P1.y < P0.y) std::swap(P0, P1);
    F2 D{P1.x - P0.x, P1.y - P0.y};
    F2 N = normalize2(F2{D.y, -D.x});
    float C = N.x * P0.x + N.y * P0.y;
    C -= 0.5f * (N.x + N.y);
    float C_sign = float_of((bits_of(C) & 0x80000000u) + 0x3f800000u);
    float k = fmax_r(1.f - C * C_sign * 0.5f, 0.f) * C_sign;
    F2 nr{k * N.x, k * N.y};
    float u = nr.x * 0.5f + 0.5f;
    float v = nr.y * 0.5f + 0.5f;
    int ix = std::min(std::max(cvt_rmi(u * 256.f), 0), 255);
    int iy = std::min(std::max(cvt_rmi(v * 256.f), 0), 255);
    const uint32_t *e = table + ((size_t)iy * 256 + ix) * words;
    for (int w = 0; w < words; ++w) out[w] = e[w];
}

// fetchVerticalTable (ras_qm_mask.h:545-560).
inline void vertical_mask(int n, float y, uint32_t *out) {
    if (n == 16) {  // 32 stacked sample rows; words (column 0, column 1)
        int32_t r = cvt_rzi(std::round(y * 32));
        uint32_t m = shr32(0xFFFFFFFFu, wsub(32, r));
        out[0] = m;
        out[1] = m;
    } else if (n == 8) {
        int32_t r = cvt_rzi(std::round(y * 16));
        uint32_t m = shr32(0xffffu, wsub(16, r));
        out[0] = m | (m << 16);
    } else {
        int32_t r = cvt_rzi(std::round(y * 64));
        uint64_t m = shr64(~0ull, wsub(64, r));
        uint32_t m0 = (uint32_t)m, m1 = (uint32_t)(m >> 32);
        out[0] = m0;
        out[1] = m1;
        out[2] = m0;
        out[3] = m1;
    }
}

// fetchVerticalTable2 (ras_qm_mask.h:562-598).
inline void vertical_mask2(int n, float y0, float y1, uint32_t *out) {
    if (n == 16) {
        int32_t s0 = std::max(wsub(32, cvt_rzi_d((double)(y0 * 32) + 0.5)), 0);
        int32_t s1 = std::max(wsub(32, cvt_rzi_d((double)(y1 * 32) + 0.5)), 0);
        uint32_t m = shr32(0xFFFFFFFFu, s0) ^ shr32(0xFFFFFFFFu, s1);
        out[0] = m;
        out[1] = m;
    } else if (n == 8) {
        int32_t s0 = wsub(16, cvt_rzi_d((double)(y0 * 16) + 0.5));
        int32_t s1 = wsub(16, cvt_rzi_d((double)(y1 * 16) + 0.5));
        s0 = std::max(s0, 0);
        s1 = std::max(s1, 0);
        uint32_t m = shr32(0xffffu, s0) ^ shr32(0xffffu, s1);
        out[0] = m | (m << 16);
    } else {
        int32_t s0 = wsub(64, cvt_rzi_d((double)(y0 * 64) + 0.5));
        int32_t s1 = wsub(64, cvt_rzi_d((double)(y1 * 64) + 0.5));
        s0 = std::max(s0, 0);
        s1 = std::max(s1, 0);
        uint64_t m = shr64(~0ull, s0) ^ shr64(~0ull, s1);
        uint32_t m0 = (uint32_t)m, m1 = (uint32_t)(m >> 32);
        out[0] = m0;
        out[1] = m1;
        out[2] = m0;
        out[3] = m1;
    }
}

// sRGB tables.  decode[k] = sRGB->linear of k/255 (GLSL srgb_to_lrgb_f,
// ms_output_32.vert.glsl:44-52, evaluated in double); thresholds[k] = the
// linear value at which the 8-bit sRGB encoding steps from k to k+1; bins
// give encode(lower edge) of 4096 equal bins of [0,1].
struct SrgbTables {
    float decode[256];
    float lin_decode[256];
    float threshold[255];
    uint8_t bin[4096];
};
SrgbTables build_srgb_tables() {
    SrgbTables t;
    auto s2l = [](double f) { return f <= 0.04045 ? f / 12.92 : std::pow((f + 0.055) / 1.055, 2.4); };
    for (int k = 0; k < 256; ++k) {
        t.decode[k] = (float)s2l(k / 255.0);
        t.lin_decode[k] = (float)k * (1.f / 255.f);
    }
    for (int k = 0; k < 255; ++k) t.threshold[k] = (float)s2l((k + 0.5) / 255.0);
    for (int b = 0; b < 4096; ++b) {
        float lo = (float)b * (1.f / 4096.f);
        int c = 0;
        while (c < 255 && lo >= t.threshold[c]) ++c;
        t.bin[b] = (uint8_t)c;
    }
    return t;
}

// --------------------------------------------------------------- result --
struct Int2 {
    int32_t x, y;
};
struct Int4 {
    int32_t x, y, z, w;
};

}  // namespace

struct orc_result {
    int width = 0, height = 0, samples = 8, words = 1;
    spr_element_number counts{};
    std::vector<F2> tvertex;
    std::vector<uint8_t> path_visible;
    std::vector<int32_t> curve_count;
    std::vector<Int2> entries;
    std::vector<int32_t> key;
    std::vector<uint32_t> pid;
    std::vector<int8_t> wn;
    std::vector<uint32_t> mask;
    std::vector<int32_t> perm;
    std::vector<int32_t> skey;
    std::vector<int8_t> wn_scan;
    std::vector<uint32_t> merged_mask;
    std::vector<Int4> draw;
    std::vector<uint8_t> image;
    // for the differentiable reference: per fragment its chord in cell
    // units (q0x, q0y, q1x, q1y) and left mask; per draw item its path; per
    // merged fragment its first sorted position
    std::vector<float> chord;
    std::vector<uint32_t> lmask;
    std::vector<uint32_t> item_path;
    std::vector<int64_t> heads;
    std::vector<uint8_t> reversed;
    std::vector<uint32_t> curve_vpos;
    std::vector<uint32_t> curve_type;
    std::vector<float> curve_w;
    double stage_ms[SPR_STAGE_COUNT_] = {};
};

namespace {

struct Scene {
    uint32_t P, C, V;
    std::vector<F2> vertex;  // after unifyCurveVertexOrder
    std::vector<uint8_t> reversed;
    const spr_scene_view *view;
};

// unifyCurveVertexOrder (ras_base.cpp:523-569): compare the first and last
// control points by their float bit patterns as uint32 and reverse the curve
// unless (y_first, x_first) < (y_last, x_last).
void unify(Scene &s) {
    const spr_scene_view *v = s.view;
    s.vertex.resize(s.V);
    std::memcpy(s.vertex.data(), v->vertex, sizeof(F2) * s.V);
    s.reversed.assign(s.C, 0);
    for (uint32_t i = 0; i < s.C; ++i) {
        int vn = v->curve_type[i] & 7;
        uint32_t p = v->curve_vertex_pos[i];
        F2 vf = s.vertex[p], vl = s.vertex[p + vn - 1];
        uint32_t ixf = bits_of(vf.x), ixl = bits_of(vl.x), iyf = bits_of(vf.y), iyl = bits_of(vl.y);
        if (iyf < iyl || (iyf == iyl && ixf < ixl)) {
            s.reversed[i] = 0;
        } else {
            s.reversed[i] = 1;
            for (int k = 0; k < vn / 2; ++k) std::swap(s.vertex[p + k], s.vertex[p + vn - k - 1]);
        }
    }
}

int validate(const spr_scene_view *v) {
    if (!v->vertex || !v->curve_vertex_pos || !v->curve_type || !v->curve_path_id ||
        !v->path_fill_rule || !v->path_fill_rgba || !v->vertex_path_id)
        return SPR_ERR_INVALID_ARG;
    uint32_t last = 0;
    for (uint32_t i = 0; i < v->n_curves; ++i) {
        int t = v->curve_type[i];
        if (t != kLinear && t != kQuad && t != kCubic && t != kRational) return SPR_ERR_INVALID_SCENE;
        if (t == kRational && !v->curve_arc_w) return SPR_ERR_INVALID_SCENE;
        if ((uint64_t)v->curve_vertex_pos[i] + (t & 7) > v->n_vertices) return SPR_ERR_INVALID_SCENE;
        uint32_t p = v->curve_path_id[i];
        if (p >= v->n_paths || p < last) return SPR_ERR_INVALID_SCENE;
        last = p;
    }
    for (uint32_t i = 0; i < v->n_vertices; ++i)
        if (v->vertex_path_id[i] >= v->n_paths) return SPR_ERR_INVALID_SCENE;
    return SPR_OK;
}

// ---------------------------------------------------- stage 3: transform --
// k_transformVertex (cu:36-105), preceded by the optional per-path affine.
void stage_transform(const Scene &s, const orc_config &cfg, orc_result &r, int threads, float pass_dy) {
    const spr_scene_view *v = s.view;
    float m[16];
    if (cfg.has_transform) {
        std::memcpy(m, cfg.transform, sizeof(m));
    } else {
        for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.f : 0.f;
    }
    const float w = (float)cfg.width, h = (float)cfg.height;
    const float z = (float)std::min(cfg.width, cfg.height);
    const float cutoff = -z * 0.5f;
    r.tvertex.resize(s.V);
    std::vector<std::atomic<uint32_t>> aflags(s.P);
    for (auto &a : aflags) a.store(0);
    parallel_for(threads, s.V, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            F2 p = s.vertex[i];
            uint32_t pid = v->vertex_path_id[i];
            if (v->path_affine) {
                const float *A = v->path_affine + 6 * (size_t)pid;
                float x = A[0] * p.x + A[2] * p.y + A[4];
                float y = A[1] * p.x + A[3] * p.y + A[5];
                p = F2{x, y};
            }
            float iv[4] = {p.x, p.y, 0.f, 1.f};
            float ov[4];
            for (int row = 0; row < 4; ++row) {
                const float *mr = m + 4 * row;
                ov[row] = mr[0] * iv[0] + mr[1] * iv[1] + mr[2] * iv[2] + mr[3] * iv[3];
            }
            ov[0] /= ov[3];
            ov[1] /= ov[3];
            ov[2] /= ov[3];
            if (ov[2] < cutoff) ov[2] = cutoff;
            float w2 = w * .5f, h2 = h * .5f;
            ov[0] = (ov[0] - w2) * z / (ov[2] + z) + w2;
            ov[1] = (ov[1] - h2) * z / (ov[2] + z) + h2;
            if (pass_dy != 0.f) ov[1] = ov[1] - pass_dy;
            int xf = ov[0] < 0 ? 0 : (ov[0] <= w ? 1 : 2);
            int yf = ov[1] < 0 ? 0 : (ov[1] <= h ? 1 : 2);
            uint32_t bit;
            switch ((yf << 4) | xf) {
            case 0x00: bit = 1u << 0; break;
            case 0x01: bit = 1u << 1; break;
            case 0x02: bit = 1u << 2; break;
            case 0x10: bit = 1u << 3; break;
            case 0x11: bit = (1u << 0) | (1u << 7); break;
            case 0x12: bit = 1u << 4; break;
            case 0x20: bit = 1u << 5; break;
            case 0x21: bit = 1u << 6; break;
            default: bit = 1u << 7; break;
            }
            aflags[pid].fetch_or(bit, std::memory_order_relaxed);
            if (std::floor(ov[0]) == ov[0]) ov[0] = ov[0] - 1.f / 256.f;
            r.tvertex[i] = F2{ov[0], ov[1]};
        }
    });
    // PATH_VISIBLE (ras_define.h:113-127): some vertex must lie outside each
    // of the four one-sided exclusion regions.
    r.path_visible.resize(s.P);
    for (uint32_t p = 0; p < s.P; ++p) {
        uint32_t f = aflags[p].load();
        bool vis = (f & 0xF8u) && (f & 0x6Bu) && (f & 0x1Fu) && (f & 0xD6u);
        r.path_visible[p] = vis ? 1 : 0;
    }
}

// ------------------------------------------ stages 4-6: intersections --
struct CurveGeom {
    int type;
    float w;
    float px[4], py[4];
    int n_pieces;
    float tcut[5];
};

// Monotonize (k_make_intersection_0, ras_cut.h:1322-1472): cut points where
// dx/dt or dy/dt vanish, insertion-sorted, then t = 1 appended.
void monotonize(CurveGeom &g, bool visible) {
    int n = 0;
    float q[5] = {0, 0, 0, 0, 0};
    if (visible) {
        for (int c = 0; c < 2; ++c) {
            const float *P = c == 0 ? g.px : g.py;
            switch (g.type) {
            case kQuad: {
                float b = (P[0] - P[1]) + (P[2] - P[1]);
                if (!(std::fabs(b) < 1e-6f)) {
                    float t = (P[0] - P[1]) / b;
                    if (t > 0.f && t < 1.f) q[n++] = t;
                }
                break;
            }
            case kCubic: {
                float r0 = 0.f, r1 = 0.f;
                solve_quad_eq((P[3] - P[0]) + 3.f * (P[1] - P[2]), 2.f * ((P[0] - P[1]) + (P[2] - P[1])),
                              P[1] - P[0], &r0, &r1);
                if (r0 > 0.f && r0 < 1.f) q[n++] = r0;
                if (r1 > 0.f && r1 < 1.f && r1 != r0) q[n++] = r1;
                break;
            }
            case kRational: {
                float w0 = 1.f, w1 = g.w, w2 = 1.f;
                float p0 = w0 * P[0], p1 = w1 * P[1], p2 = w2 * P[2];
                float pw01 = p0 * w1 - p1 * w0;
                float pw12 = p1 * w2 - p2 * w1;
                float pw20 = p2 * w0 - p0 * w2;
                float r0 = 0.f, r1 = 0.f;
                solve_quad_eq(pw01 + pw12 + pw20, -(2.f * pw01 + pw20), pw01, &r0, &r1);
                if (r0 > 0.f && r0 < 1.f) q[n++] = r0;
                if (r1 > 0.f && r1 < 1.f && r1 != r0) q[n++] = r1;
                break;
            }
            default:
                break;
            }
        }
        for (int i = 1; i < n; ++i) {  // stable insertion sort, strict <
            float t = q[i];
            int j = i - 1;
            while (j >= 0 && t < q[j]) {
                q[j + 1] = q[j];
                --j;
            }
            q[j + 1] = t;
        }
        q[n++] = 1.f;
    }
    g.n_pieces = n;
    for (int i = 0; i < 5; ++i) g.tcut[i] = q[i];
}

// d_get_xy_begin_end + d_udpate_cut_range (ras_cut.h:670-777): cell lines
// crossed by the piece v0 -> v1, clamped to [0, (dim & ~1) + 2].
struct CutRange {
    int xb, xe, yb, ye, nx, ny;
    float dx, dy;
};
inline CutRange cut_range(F2 v0, F2 v1, int W, int H) {
    CutRange c;
    if (v0.x <= v1.x) {
        c.xb = floor2(v0.x) + 2;
        c.xe = floor2(v1.x);
        c.dx = 2.f;
    } else {
        c.xb = floor2(v1.x) + 2;
        c.xe = floor2(v0.x);
        c.dx = -2.f;
    }
    if (v0.y <= v1.y) {
        c.yb = floor2(v0.y) + 2;
        c.ye = floor2(v1.y);
        c.dy = 2.f;
    } else {
        c.yb = floor2(v1.y) + 2;
        c.ye = floor2(v0.y);
        c.dy = -2.f;
    }
    const int xmax = (W & ~1) + 2, ymax = (H & ~1) + 2;
    auto clampi = [](int x, int lo, int hi) { return std::min(std::max(x, lo), hi); };
    if ((c.xb < 0 && c.xe < 0) || (c.xb > xmax && c.xe > xmax) || (c.xb > c.xe)) {
        c.nx = 0;
    } else {
        c.xb = clampi(c.xb, 0, xmax);
        c.xe = clampi(c.xe, 0, xmax);
        c.nx = std::max((c.xe - c.xb) / 2 + 1, 0);
    }
    if ((c.yb < 0 && c.ye < 0) || (c.yb > ymax && c.ye > ymax) || (c.yb > c.ye)) {
        c.ny = 0;
    } else {
        c.yb = clampi(c.yb, 0, ymax);
        c.ye = clampi(c.ye, 0, ymax);
        c.ny = std::max((c.ye - c.yb) / 2 + 1, 0);
    }
    return c;
}

// k_make_intersection_impl_0 (ras_cut.h:780-834).
int count_curve(const CurveGeom &g, int W, int H) {
    F2 v0{g.px[0], g.py[0]};
    int p = 0;
    for (int i = 0; i < g.n_pieces; ++i) {
        float t1 = g.tcut[i];
        F2 v1{curve_coord(g.type, g.w, g.px, t1), curve_coord(g.type, g.w, g.py, t1)};
        CutRange c = cut_range(v0, v1, W, H);
        p += 1 + c.nx + c.ny;
        v0 = v1;
    }
    return p;
}

// Root of curve coordinate P(t) = c on [tmin, tmax] (ras_cut.h:1020-1225):
// lines by one division, quadratics and rationals by solveQuadBezierQM,
// cubics by 24 bisection steps, falling back to tmin when the final residual
// exceeds one pixel.
inline float solve_crossing(const CurveGeom &g, const float *P, float c, float tmin, float tmax) {
    switch (g.type) {
    case kLinear: {
        // Rasterizer::min / max (ras_device_func.h:20-28): plain ternaries.
        float t = (c - P[0]) * safe_rcp(P[1] - P[0]);
        t = t > tmin ? t : tmin;
        return t < tmax ? t : tmax;
    }
    case kQuad:
        return solve_quad_bezier(P[0], P[1], P[2], c, tmin, tmax);
    case kRational:
        return solve_quad_bezier(P[0] - c, (P[1] - c) * g.w, P[2] - c, 0.f, tmin, tmax);
    default: {
        float t0 = tmin, t1 = tmax;
        float vt0 = curve_coord(kCubic, 0.f, P, t0);
        float ts = t0;
        if (vt0 != c) {
            float raw_t0 = t0;
            float last = 0.f;
            for (int it = 0; it < 24; ++it) {
                float tm = (t0 + t1) * .5f;
                float vtm = curve_coord(kCubic, 0.f, P, tm);
                ts = tm;
                last = vtm;
                if ((int32_t)(bits_of(vtm - c) ^ bits_of(vt0 - c)) >= 0) {
                    t0 = tm;
                    vt0 = vtm;
                } else {
                    t1 = tm;
                }
            }
            if (std::fabs(last - c) > 1.f) ts = raw_t0;
        }
        return ts;
    }
    }
}

// k_make_intersection_impl_1 (ras_cut.h:837-1241): per monotone piece, the
// piece start followed by every x-line and y-line crossing, merged by t.  The
// low two bits of t carry flags: bit 0 = crossing side (1 = horizontal line),
// bit 1 = piece end; equal t values OR their flags into both entries.
void emit_curve(const CurveGeom &g, int32_t cid, int W, int H, Int2 *out) {
    float t0_ms = 0.f;
    F2 v0{g.px[0], g.py[0]};
    int p = 0;
    for (int ms = 0; ms < g.n_pieces; ++ms) {
        float traw = g.tcut[ms];
        F2 v1{curve_coord(g.type, g.w, g.px, traw), curve_coord(g.type, g.w, g.py, traw)};
        uint32_t tb = bits_of(traw) & 0xFFFFFFFCu;
        float t1_ms = (std::floor(v1.x) == v1.x) ? float_of(tb | 2u) : float_of(tb | 3u);
        CutRange cr = cut_range(v0, v1, W, H);
        int nx = cr.nx, ny = cr.ny;
        const int n_loop = nx + ny + 1;
        float x = (float)(cr.dx < 0.f ? cr.xe : cr.xb);
        float y = (float)(cr.dy < 0.f ? cr.ye : cr.yb);
        float slot[2] = {t0_ms, t0_ms};
        uint32_t last = bits_of(-1.f);
        for (int i = -1; i < n_loop; ++i) {
            float t_solve = 0.f, c = 0.f, t_min;
            int side = 0;
            float ntx = slot[0], nty = slot[1];
            if (i == -1) {
                t_min = ntx;
                if (nx == 0) {
                    side = 0;
                    t_solve = 2.f;
                } else if (ny == 0) {
                    side = 1;
                    t_solve = 2.f;
                } else {
                    side = 0;
                    nx--;
                    c = x;
                    x += cr.dx;
                }
            } else if (ntx <= nty) {
                t_min = ntx;
                side = 0;
                if (nx > 0) {
                    nx--;
                    c = x;
                    x += cr.dx;
                } else {
                    t_solve = 2.f;
                }
            } else {
                t_min = nty;
                side = 1;
                if (ny > 0) {
                    ny--;
                    c = y;
                    y += cr.dy;
                } else {
                    t_solve = 2.f;
                }
            }
            if (i >= 0) {
                uint32_t ob = bits_of(t_min);
                if ((ob & 0xFFFFFFFCu) == (last & 0xFFFFFFFCu)) {
                    ob |= last;
                    out[p - 1] = Int2{cid, (int32_t)ob};
                }
                out[p] = Int2{cid, (int32_t)ob};
                last = ob;
                p++;
            }
            if (t_solve < 2.f) t_solve = solve_crossing(g, side ? g.py : g.px, c, t_min, t1_ms);
            slot[side] = float_of((bits_of(t_solve) & 0xFFFFFFFCu) | (uint32_t)side);
        }
        t0_ms = t1_ms;
        v0 = v1;
    }
}

void load_geom(const Scene &s, const orc_result &r, uint32_t i, CurveGeom &g) {
    const spr_scene_view *v = s.view;
    g.type = v->curve_type[i];
    g.w = (g.type == kRational) ? v->curve_arc_w[i] : 0.f;
    uint32_t p0 = v->curve_vertex_pos[i];
    int n = g.type & 7;
    for (int j = 0; j < 4; ++j) {
        if (j < n) {
            g.px[j] = r.tvertex[p0 + j].x;
            g.py[j] = r.tvertex[p0 + j].y;
        } else {
            g.px[j] = 0.f;
            g.py[j] = 0.f;
        }
    }
}

// ------------------------------------------------ stage 7: fragments --
struct FragCtx {
    const Scene *s;
    const orc_result *r;
    const uint32_t *table;
    int W, H, S, words;
};

// k_gen_fragment_and_stencil_mask (cu:112-441) for entry i.
void make_fragment(const FragCtx &fc, int64_t i, int64_t nf, int32_t *key, uint32_t *pidw, int8_t *wn,
                   uint32_t *mask, float *chord, uint32_t *lmask) {
    const orc_result &r = *fc.r;
    const spr_scene_view *v = fc.s->view;
    Int2 e0 = r.entries[i];
    Int2 e1 = (i + 1) != nf ? r.entries[i + 1] : Int2{-1, 0x3f800000};
    int f0 = e0.y & 1, f1 = e1.y & 1;
    float t0 = float_of((uint32_t)e0.y & 0xFFFFFFFCu);
    float t1 = float_of((uint32_t)e1.y & 0xFFFFFFFCu);
    if (t0 < 0) t0 = 0.f;
    if (t1 < 0) t1 = 0.f;
    if (t0 == 0.f || t0 == 1.f) f0 = 1;
    if (t1 == 0.f || t1 == 1.f) f1 = 1;
    int32_t cid = e0.x;
    uint32_t pathid = v->curve_path_id[cid];
    int32_t yx = (int32_t)0xFFFEFFFEu;
    if (e0.x != e1.x) t1 = 1.f;
    int wnchg = 0, swn = 0;
    for (int w = 0; w < fc.words; ++w) mask[w] = 0;
    for (int w = 0; w < fc.words; ++w) lmask[w] = 0;
    for (int k = 0; k < 4; ++k) chord[k] = 0.f;
    if (t0 < t1) {
        CurveGeom g;
        load_geom(*fc.s, r, (uint32_t)cid, g);
        float tt[2] = {t0, t1};
        F2 cp[2];
        for (int k = 0; k < 2; ++k) {
            float fi = k / 1.f;
            float t = (1 - fi) * tt[0] + fi * tt[1];
            cp[k] = F2{curve_coord(g.type, g.w, g.px, t), curve_coord(g.type, g.w, g.py, t)};
        }
        bool rev = fc.s->reversed[cid] != 0;
        F2 vf = rev ? cp[1] : cp[0];
        F2 vl = rev ? cp[0] : cp[1];
        int sf = rev ? f1 : f0;
        int sl = rev ? f0 : f1;
        int rx = floor2((vf.x + vl.x) * 0.5f);
        int ry = floor2((vf.y + vl.y) * 0.5f);
        int px = std::min(std::max(rx, -2), (int)(((uint32_t)fc.W & 0xFFFFFFFEu) + 2));
        int py = std::min(std::max(ry, -2), (int)(((uint32_t)fc.H & 0xFFFFFFFEu) + 2));
        uint32_t ys = (uint32_t)(py + 0x7FFF) << 16;
        uint32_t xs = (uint32_t)(px + 0x7FFF) & 0xFFFFu;
        if ((uint32_t)ry < (uint32_t)fc.H) yx = (int32_t)(ys | xs);
        int wy = py + 1;
        if (vf.y == vl.y) {
            swn = 0;
        } else if (vf.y <= wy && wy < vl.y) {
            swn = -1;
        } else if (vl.y <= wy && wy < vf.y) {
            swn = 1;
        }
        if (vf.y < vl.y) {
            wnchg = -1;
        } else if (vf.y > vl.y) {
            wnchg = 1;
        } else {
            wnchg = (vf.x < vl.x) ? 1 : -1;
        }
        F2 vleft{0, 0}, vright{0, 0};
        int left_flag = 1;
        if (vf.x < vl.x) {
            vleft = vf;
            vright = vl;
            left_flag = sf;
        } else if (vf.x > vl.x) {
            vleft = vl;
            vright = vf;
            left_flag = sl;
        } else if (vf.x < px + 1) {
            if (sf == 0) {
                vleft = vf;
                vright = vl;
                left_flag = 0;
            } else if (sl == 0) {
                vleft = vl;
                vright = vf;
                left_flag = 0;
            }
        }
        uint32_t lm[4] = {0, 0, 0, 0};
        if (left_flag == 0) {
            vertical_mask(fc.S, (vleft.y - py) * .5f, lm);
            if (vleft.y <= py + 1) {
                if (vleft.y >= vright.y) wnchg = -wnchg;
            } else {
                if (vleft.y < vright.y) wnchg = -wnchg;
                for (int w = 0; w < 4; ++w) lm[w] = ~lm[w];
            }
        }
        F2 base{(float)px, (float)py};
        F2 c0{(cp[0].x - base.x) * .5f, (cp[0].y - base.y) * .5f};
        F2 c1{(cp[1].x - base.x) * .5f, (cp[1].y - base.y) * .5f};
        uint32_t vm[4], tm[4];
        vertical_mask2(fc.S, c0.y, c1.y, vm);
        fetch_pixel_table(fc.table, fc.words, c0, c1, tm);
        for (int w = 0; w < fc.words; ++w) mask[w] = (tm[w] & vm[w]) ^ lm[w];
        for (int w = 0; w < fc.words; ++w) lmask[w] = lm[w];
        chord[0] = c0.x;
        chord[1] = c0.y;
        chord[2] = c1.x;
        chord[3] = c1.y;
    }
    key[i] = yx;
    pidw[i] = pathid | ((uint32_t)wnchg << 30);
    wn[i] = (int8_t)swn;
}

// Decoding of a cell key (cu:482-483): int16 fields offset by 0x7FFF.
inline int16_t key_x(uint32_t k) { return (int16_t)(uint16_t)((k & 0xFFFFu) - 0x7FFFu); }
inline int16_t key_y(uint32_t k) { return (int16_t)(uint16_t)((k >> 16) - 0x7FFFu); }

// Decoded channel value as an exact 2^-36 fixed-point integer.
inline int64_t fixed36(float d) { return (int64_t)(d * 68719476736.0f); }

// Gradient paints, restating the renderer's evaluation of the reference's
// GL shaders (ms_output_32.vert.glsl calc_color, ms_output_32.frag.glsl):
// the pixel centre back through the reverse transform, the entry's 2x3 map
// at both ends of the item's row interpolated to the pixel, the focal-point
// ratio, the ramp linearly filtered (texels decoded by `dec`).
inline void grad_coord(const float *rev, const float *e, float x, float y, float &gx, float &gy) {
    const float rdx = (rev[0] * x + rev[3] * y) + rev[6];
    const float rdy = (rev[1] * x + rev[4] * y) + rev[7];
    const float rdz = (rev[2] * x + rev[5] * y) + rev[8];
    const float k = rev[12] / rdz;
    const float ox = rev[9] + k * rdx, oy = rev[10] + k * rdy;
    gx = (ox * e[0] + oy * e[1]) + e[2];
    gy = (ox * e[3] + oy * e[4]) + e[5];
}

void gradient_colour(const orc_config &cfg, const float *rev, const float *dec, const float *lin, uint32_t entry,
                     int x0, int w, int X, int Y, float &sr, float &sg, float &sb, float &sa) {
    float e[12];
    std::memcpy(e, cfg.grad_table + 12 * (size_t)entry, sizeof(e));
    const float yr = (float)Y + 0.5f;
    float g0x, g0y, g1x, g1y;
    grad_coord(rev, e, (float)x0, yr, g0x, g0y);
    grad_coord(rev, e, (float)(x0 + w), yr, g1x, g1y);
    const float t = ((float)X + 0.5f - (float)x0) / (float)w;
    const float gx = g0x * (1.f - t) + g1x * t, gy = g0y * (1.f - t) + g1y * t;
    const float dx = gx - e[8], dy = gy - e[9];
    const float A = dx * dx + dy * dy, B = dx * e[8] + dy * e[9];
    const float den = std::sqrt(B * B + A * e[10]) - B;
    const float c = std::min(A * (den > 1e-6f ? 1.f / den : 0.f), 1.f);
    int32_t p;
    std::memcpy(&p, &e[6], 4);
    const float pos = c * (e[7] * 1024.f);
    const int i0 = (int)std::floor(pos);
    const float f = pos - (float)i0;
    const int row = p >> 10, col = std::min((p & 1023) + i0, 1023), col1 = std::min(col + 1, 1023);
    const uint32_t t0 = cfg.grad_ramp[row * 1024 + col], t1 = cfg.grad_ramp[row * 1024 + col1];
    const float u = 1.f - f;
    sr = dec[t0 & 0xFF] * u + dec[t1 & 0xFF] * f;
    sg = dec[(t0 >> 8) & 0xFF] * u + dec[(t1 >> 8) & 0xFF] * f;
    sb = dec[(t0 >> 16) & 0xFF] * u + dec[(t1 >> 16) & 0xFF] * f;
    sa = lin[t0 >> 24] * u + lin[t1 >> 24] * f;
}

inline uint32_t enc_lin(float v) {
    float c = fmin_r(fmax_r(v, 0.f), 1.f);
    return (uint32_t)cvt_rzi(c * 255.f + 0.5f);
}
inline uint32_t enc_srgb(const SrgbTables &t, float v) {
    float c = fmin_r(fmax_r(v, 0.f), 1.f);
    int b = std::min(cvt_rzi(c * 4096.f), 4095);
    uint32_t k = t.bin[b];
    if (k < 255 && c >= t.threshold[k]) ++k;
    return k;
}

}  // namespace

// ================================================================= API ==
namespace {

// One frame (pass < 0), or pass `pass` of a 256-sample frame (cfg.samples
// 32, the pass's samples and shift; the resolve adds its fixed-point sample
// sums, 4 per pixel, to `sums` instead of writing the image).
int run_frame(const spr_scene_view *scene, const orc_config &cfg, int pass, orc_result &r, int64_t *sums) {
    if (cfg.width < 1 || cfg.height < 1 || cfg.width > 4096 || cfg.height > 4096) return SPR_ERR_INVALID_ARG;
    if (cfg.samples != 8 && cfg.samples != 16 && cfg.samples != 32) return SPR_ERR_INVALID_ARG;
    int rc = validate(scene);
    if (rc) return rc;
    int threads = cfg.threads > 0 ? cfg.threads : (int)std::max(1u, std::thread::hardware_concurrency());
    const int stop = cfg.stop_after < 0 ? SPR_STAGE_COUNT_ : cfg.stop_after;
    r.width = cfg.width;
    r.height = cfg.height;
    r.samples = cfg.samples;
    r.words = cfg.samples / 8;
    const int W = cfg.width, H = cfg.height, S = cfg.samples, WORDS = r.words;

    Scene s;
    s.view = scene;
    s.P = scene->n_paths;
    s.C = scene->n_curves;
    s.V = scene->n_vertices;
    r.counts.path = (int32_t)s.P;
    r.counts.curve = (int32_t)s.C;
    r.counts.vertex = (int32_t)s.V;
    unify(s);
    r.reversed = s.reversed;

    using clk = std::chrono::steady_clock;
    auto t_prev = clk::now();
    auto lap = [&](int stage) {
        auto now = clk::now();
        r.stage_ms[stage] += std::chrono::duration<double, std::milli>(now - t_prev).count();
        t_prev = now;
    };

    // -- stage 3 ---------------------------------------------------------
    stage_transform(s, cfg, r, threads, pass >= 0 ? pass_shift_256(pass) : 0.f);
    lap(SPR_STAGE_TVERTEX);
    if (stop <= SPR_STAGE_PATH_VISIBLE) return SPR_OK;

    // -- stages 4-5: monotonize + count + exclusive scan --------------------
    std::vector<CurveGeom> geoms(s.C);
    r.curve_count.assign(s.C, 0);
    parallel_for(threads, s.C, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            CurveGeom &g = geoms[i];
            load_geom(s, r, (uint32_t)i, g);
            monotonize(g, r.path_visible[s.view->curve_path_id[i]] != 0);
            r.curve_count[i] = count_curve(g, W, H);
        }
    });
    std::vector<int64_t> offs(s.C + 1, 0);
    for (uint32_t i = 0; i < s.C; ++i) offs[i + 1] = offs[i] + r.curve_count[i];
    const int64_t nf = offs[s.C];
    if (nf > INT32_MAX) return SPR_ERR_CAPACITY_EXCEEDED;
    r.counts.curve_fragment = (int32_t)nf;
    lap(SPR_STAGE_CURVE_COUNT);
    if (stop <= SPR_STAGE_CURVE_COUNT) return SPR_OK;

    // -- stage 6: emit ------------------------------------------------------
    r.entries.resize(nf);
    parallel_for(threads, s.C, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i)
            if (r.curve_count[i]) emit_curve(geoms[i], (int32_t)i, W, H, r.entries.data() + offs[i]);
    });
    geoms.clear();
    geoms.shrink_to_fit();
    lap(SPR_STAGE_INTERSECTION);
    if (stop <= SPR_STAGE_INTERSECTION) return SPR_OK;

    // -- stage 7: fragments + boundary masks ---------------------------------
    // (the table is built once per renderer in the reference; not timed here)
    auto t_table = clk::now();
    std::vector<uint32_t> table = pass >= 0 ? build_pass_mask_table_256(pass) : build_mask_table(S);
    t_prev += clk::now() - t_table;
    r.key.resize(nf);
    r.pid.resize(nf);
    r.wn.resize(nf);
    r.mask.resize(nf * WORDS);
    r.chord.resize(4 * nf);
    r.lmask.resize(nf * WORDS);
    FragCtx fc{&s, &r, table.data(), W, H, S, WORDS};
    parallel_for(threads, nf, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i)
            make_fragment(fc, i, nf, r.key.data(), r.pid.data(), r.wn.data(), r.mask.data() + i * WORDS,
                          r.chord.data() + 4 * i, r.lmask.data() + i * WORDS);
    });
    lap(SPR_STAGE_FRAG_MASK);
    if (stop <= SPR_STAGE_FRAG_MASK) return SPR_OK;

    // -- stage 8: stable sort by signed key within each path segment ---------
    // (SegSortPairsFromIndices, segmentedsort_ext.cuh:216-268; segments are
    // the per-path ranges written at cu:422-439).
    r.perm.resize(nf);
    for (int64_t i = 0; i < nf; ++i) r.perm[i] = (int32_t)i;
    std::vector<int64_t> seg_start;
    seg_start.reserve(s.P + 1);
    {
        int64_t i = 0;
        while (i < nf) {
            seg_start.push_back(i);
            uint32_t p = r.pid[i] & 0x3FFFFFFFu;
            while (i < nf && (r.pid[i] & 0x3FFFFFFFu) == p) ++i;
        }
        seg_start.push_back(nf);
    }
    const int64_t nseg = (int64_t)seg_start.size() - 1;
    parallel_for(threads, nseg, [&](int64_t b, int64_t e) {
        for (int64_t sg = b; sg < e; ++sg) {
            auto first = r.perm.begin() + seg_start[sg], last = r.perm.begin() + seg_start[sg + 1];
            std::stable_sort(first, last, [&](int32_t a, int32_t c) { return r.key[a] < r.key[c]; });
        }
    });
    r.skey.resize(nf);
    for (int64_t i = 0; i < nf; ++i) r.skey[i] = r.key[r.perm[i]];
    lap(SPR_STAGE_SORT_PERM);
    if (stop <= SPR_STAGE_SORT_KEY) return SPR_OK;

    // -- stages 9-10: shuffle + global int8 exclusive scan (cu:444-456, 1099) --
    r.wn_scan.resize(nf);
    {
        uint8_t acc = 0;
        for (int64_t i = 0; i < nf; ++i) {
            r.wn_scan[i] = (int8_t)acc;
            acc = (uint8_t)(acc + (uint8_t)r.wn[r.perm[i]]);
        }
    }
    lap(SPR_STAGE_WN_SCAN);
    if (stop <= SPR_STAGE_WN_SCAN) return SPR_OK;

    // -- stages 11-12: merged-fragment / span flags + inclusive scans
    // (k_mark_merged_fragment_and_span, cu:462-535; cu:1139-1157).  The path
    // id at a sorted position equals the raw one: the sort never moves an
    // entry across a path segment.
    std::vector<uint8_t> fflag(nf), sflag(nf);
    const uint8_t *rule = scene->path_fill_rule;
    parallel_for(threads, nf, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            uint32_t k1 = (uint32_t)r.skey[i];
            int x1 = key_x(k1), y1 = key_y(k1);
            bool oob = x1 < 0 || y1 < 0 || x1 >= W || y1 >= H;
            if (i == 0) {
                fflag[i] = oob ? 0 : 1;
                sflag[i] = 0;
                continue;
            }
            uint32_t p0 = r.pid[i - 1] & 0x3FFFFFFFu, p1 = r.pid[i] & 0x3FFFFFFFu;
            uint8_t fr = rule[p1];
            uint32_t k0 = (uint32_t)r.skey[i - 1];
            int x0 = key_x(k0), y0 = key_y(k0);
            if (oob)
                fflag[i] = 0;
            else
                fflag[i] = (p0 != p1 || k0 != k1) ? 1 : 0;
            int8_t w = r.wn_scan[i];
            bool wf = (fr == 0 && w != 0) || (fr == 1 && (w & 1));
            sflag[i] = (y0 == y1 && (x0 + 2) < x1 && p0 == p1 && wf) ? 1 : 0;
        }
    });
    std::vector<int32_t> fidx(nf), sidx(nf);
    int64_t nm = 0, ns = 0;
    for (int64_t i = 0; i < nf; ++i) {
        nm += fflag[i];
        fidx[i] = (int32_t)nm;
    }
    for (int64_t i = 0; i < nf; ++i) {
        ns += sflag[i];
        sidx[i] = (int32_t)ns;
    }
    r.counts.merged_fragment = (int32_t)nm;
    r.counts.span = (int32_t)ns;

    // -- stage 13: merged masks (k_gen_stencil_cuda_sm, cu:554-722, with the
    // block-boundary fix-up of cu:724-786 folded in: every group is summed in
    // one pass).  Per mask bit j: 8-bit lanes counting +/- boundary crossings
    // on top of the scanned winding number, 7-bit result, then the fill rule.
    r.merged_mask.assign(nm * WORDS, 0);
    std::vector<int64_t> heads(nm);
    for (int64_t i = 0; i < nf; ++i)
        if (fflag[i]) heads[fidx[i] - 1] = i;
    parallel_for(threads, nm, [&](int64_t b, int64_t e) {
        for (int64_t g = b; g < e; ++g) {
            int64_t h = heads[g];
            uint32_t kh = (uint32_t)r.skey[h];
            uint32_t ph = r.pid[h] & 0x3FFFFFFFu;
            int32_t w0 = r.wn_scan[h];
            uint32_t init_pos = w0 < 0 ? 0u : 0x01010101u * (uint32_t)w0;
            uint32_t init_neg = w0 < 0 ? 0x01010101u * (uint32_t)(-w0) : 0u;
            uint32_t pos[4][8], neg[4][8];
            for (int w = 0; w < 4; ++w)
                for (int bb = 0; bb < 8; ++bb) {
                    pos[w][bb] = init_pos;
                    neg[w][bb] = init_neg;
                }
            for (int64_t j = h; j < nf && (uint32_t)r.skey[j] == kh && (r.pid[j] & 0x3FFFFFFFu) == ph; ++j) {
                int32_t raw = r.perm[j];
                int32_t chg = (int32_t)r.pid[raw] >> 30;
                if (chg == 0) continue;
                const uint32_t *m = r.mask.data() + (int64_t)raw * WORDS;
                for (int w = 0; w < WORDS; ++w)
                    for (int bb = 0; bb < 8; ++bb) {
                        uint32_t a = (m[w] >> bb) & 0x01010101u;
                        if (chg > 0)
                            pos[w][bb] += a;
                        else
                            neg[w][bb] += a;
                    }
            }
            const int fr = rule[ph];
            for (int w = 0; w < WORDS; ++w) {
                uint32_t ret = 0;
                for (int bb = 0; bb < 8; ++bb) {
                    uint32_t wv = (0x80808080u + pos[w][bb] - neg[w][bb]) & 0x7f7f7f7fu;
                    if (fr == 0) {
                        wv |= wv >> 4;
                        wv |= wv >> 2;
                        wv |= wv >> 1;
                    }
                    ret |= (wv & 0x01010101u) << bb;
                }
                r.merged_mask[g * WORDS + w] = ret;
            }
        }
    });
    lap(SPR_STAGE_MERGED_MASK);

    // -- stage 14: draw list (k_gen_gl_merged_fragment_and_span, cu:789-868) --
    r.draw.resize(nm + ns);
    r.item_path.resize(nm + ns);
    r.heads = heads;
    const uint32_t *fill = scene->path_fill_rgba;
    parallel_for(threads, nf, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            int ff = fflag[i], sfv = sflag[i];
            if (!ff && !sfv) continue;
            int32_t nfb = fidx[i] - ff, nsb = sidx[i] - sfv;
            uint32_t p = r.pid[i] & 0x3FFFFFFFu;
            uint32_t fi = fill[p];
            if (ff) {
                uint32_t k = (uint32_t)r.skey[i];
                int32_t pos = (int32_t)(((uint32_t)(int32_t)key_y(k) << 16) | (uint32_t)(int32_t)key_x(k));
                r.draw[nfb + nsb] = Int4{pos, 2, (int32_t)fi, fidx[i]};
                r.item_path[nfb + nsb] = p;
            }
            if (sfv) r.item_path[nfb + nsb + ff] = p;
            if (sfv) {
                uint32_t k0 = (uint32_t)r.skey[i - 1], k1 = (uint32_t)r.skey[i];
                int y0 = key_y(k0);
                int x0 = (int16_t)(key_x(k0) + 2);
                int x1 = key_x(k1);
                x0 = std::max(0, x0);
                int32_t pos = (int32_t)(((uint32_t)y0 << 16) | (uint32_t)x0);
                r.draw[nfb + nsb + ff] = Int4{pos, x1 - x0, (int32_t)fi, 0};
            }
        }
    });
    lap(SPR_STAGE_DRAW_LIST);
    if (stop <= SPR_STAGE_DRAW_LIST) return SPR_OK;

    // -- stage 15: coverage / colour resolve (GL draw of cu:1312-1433 with the
    // ms_output_{8,32} / output_{8,32} shaders, then the multisample resolve
    // blit of ras_base.cpp:1146-1163), restated on the CPU.  Items are applied
    // in draw-list order per pixel; each item covers pixels [x, x+w) of rows
    // y and y+1.
    auto t_tables = clk::now();
    const SrgbTables st = build_srgb_tables();
    t_prev += clk::now() - t_tables;
    const int nrows = (H + 1) / 2;
    std::vector<std::vector<int32_t>> row_items(nrows);
    for (int64_t it = 0; it < nm + ns; ++it) {
        int32_t y = (int32_t)((uint32_t)r.draw[it].x >> 16) ;
        y = (int16_t)(uint16_t)y;
        if (y >= 0 && y < H) row_items[y / 2].push_back((int32_t)it);
    }
    const int spp = cfg.ms_output ? S : 1;
    const float *dec = cfg.srgb ? st.decode : st.lin_decode;
    const float rev_identity[13] = {1.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 1.f};
    const float *rev = cfg.has_rev ? cfg.rev : rev_identity;
    r.image.assign((size_t)W * H * 4, 0);
    parallel_for(threads, nrows, [&](int64_t b, int64_t e) {
        std::vector<uint32_t> state((size_t)2 * W * spp);
        for (int64_t row = b; row < e; ++row) {
            std::fill(state.begin(), state.end(), 0xFFFFFFFFu);
            const int ybase = (int)row * 2;
            for (int32_t it : row_items[row]) {
                const Int4 d = r.draw[it];
                int x = (int16_t)(uint16_t)((uint32_t)d.x & 0xFFFFu);
                uint32_t c = (uint32_t)d.z;
                float sr = dec[c & 0xFF], sg = dec[(c >> 8) & 0xFF], sb = dec[(c >> 16) & 0xFF];
                float sa = st.lin_decode[c >> 24];
                const bool grad = cfg.grad_table != nullptr && c - 1u < cfg.n_grad;
                for (int py = 0; py < 2; ++py) {
                    int yy = ybase + py;
                    if (yy >= H) continue;
                    int xlo = std::max(x, 0), xhi = std::min(x + d.y, W);
                    for (int xx = xlo; xx < xhi; ++xx) {
                        uint32_t m = 0xFFFFFFFFu;
                        if (d.w != 0) {
                            int k = (xx - x) * 2 + py;
                            if (S == 8)
                                m = (r.merged_mask[(int64_t)(d.w - 1)] >> (8 * k)) & 0xFFu;
                            else if (S == 16)
                                m = (r.merged_mask[(int64_t)(d.w - 1) * 2 + (k >> 1)] >> (16 * (k & 1))) & 0xFFFFu;
                            else
                                m = r.merged_mask[(int64_t)(d.w - 1) * 4 + k];
                        }
                        uint32_t *px = state.data() + ((size_t)py * W + xx) * spp;
                        if (grad)
                            gradient_colour(cfg, rev, dec, st.lin_decode, c - 1u, x, d.y, xx, yy, sr, sg, sb, sa);
                        float a = sa;
                        if (!cfg.ms_output) {
                            int cnt = __builtin_popcount(S == 32 ? m : (m & ((1u << S) - 1u)));
                            a = sa * ((float)cnt / (float)S);
                            m = 1u;
                        }
                        const float om = 1.f - a;
                        for (int smp = 0; smp < spp; ++smp) {
                            if (!((m >> smp) & 1u)) continue;
                            uint32_t dv = px[smp];
                            float dr = dec[dv & 0xFF], dg = dec[(dv >> 8) & 0xFF], db = dec[(dv >> 16) & 0xFF];
                            float da = st.lin_decode[dv >> 24];
                            float orr = sr * a + dr * om;
                            float og = sg * a + dg * om;
                            float ob = sb * a + db * om;
                            float oa = a * a + da * om;
                            uint32_t er, eg, eb;
                            if (cfg.srgb) {
                                er = enc_srgb(st, orr);
                                eg = enc_srgb(st, og);
                                eb = enc_srgb(st, ob);
                            } else {
                                er = enc_lin(orr);
                                eg = enc_lin(og);
                                eb = enc_lin(ob);
                            }
                            px[smp] = er | (eg << 8) | (eb << 16) | (enc_lin(oa) << 24);
                        }
                    }
                }
            }
            for (int py = 0; py < 2; ++py) {
                int yy = ybase + py;
                if (yy >= H) continue;
                for (int xx = 0; xx < W; ++xx) {
                    // Average over the samples, exactly: every decoded value is a
                    // float >= 2^-12 (or 0), so value * 2^36 is an integer and the
                    // 64-bit sum is exact; one rounding to float at the end.
                    const uint32_t *px = state.data() + ((size_t)py * W + xx) * spp;
                    int64_t ir = 0, ig = 0, ib = 0, ia = 0;
                    for (int smp = 0; smp < spp; ++smp) {
                        uint32_t v = px[smp];
                        ir += fixed36(dec[v & 0xFF]);
                        ig += fixed36(dec[(v >> 8) & 0xFF]);
                        ib += fixed36(dec[(v >> 16) & 0xFF]);
                        ia += fixed36(st.lin_decode[v >> 24]);
                    }
                    if (sums) {
                        int64_t *q = sums + ((size_t)yy * W + xx) * 4;
                        q[0] += ir;
                        q[1] += ig;
                        q[2] += ib;
                        q[3] += ia;
                        continue;
                    }
                    const double scale = 1.0 / (68719476736.0 * (double)spp);
                    const float ar = (float)((double)ir * scale), ag = (float)((double)ig * scale);
                    const float ab = (float)((double)ib * scale), aa = (float)((double)ia * scale);
                    uint8_t *o = r.image.data() + ((size_t)yy * W + xx) * 4;
                    if (cfg.srgb) {
                        o[0] = (uint8_t)enc_srgb(st, ar);
                        o[1] = (uint8_t)enc_srgb(st, ag);
                        o[2] = (uint8_t)enc_srgb(st, ab);
                    } else {
                        o[0] = (uint8_t)enc_lin(ar);
                        o[1] = (uint8_t)enc_lin(ag);
                        o[2] = (uint8_t)enc_lin(ab);
                    }
                    o[3] = (uint8_t)enc_lin(aa);
                }
            }
        }
    });
    lap(SPR_STAGE_IMAGE);
    return SPR_OK;
}

}  // namespace

// 256 samples: 8 passes of 32 (their sample sums added exactly, then the
// resolve's averaging and encoding over all 256); the result holds the last
// pass's stages and counts.
extern "C" int orc_run(const spr_scene_view *scene, const orc_config *cfgp, orc_result **out) {
    if (!scene || !cfgp || !out) return SPR_ERR_INVALID_ARG;
    orc_result *rp = new orc_result();
    *out = rp;
    if (cfgp->samples != 256) return run_frame(scene, *cfgp, -1, *rp, nullptr);
    if (!cfgp->ms_output) return SPR_ERR_INVALID_ARG;
    if (cfgp->width < 1 || cfgp->height < 1 || cfgp->width > 4096 || cfgp->height > 4096) return SPR_ERR_INVALID_ARG;
    orc_config c = *cfgp;
    c.samples = 32;
    const int W = c.width, H = c.height;
    std::vector<int64_t> sums((size_t)W * H * 4, 0);
    double ms[SPR_STAGE_COUNT_] = {};
    for (int g = 0; g < 8; ++g) {
        *rp = orc_result();
        const int rc = run_frame(scene, c, g, *rp, sums.data());
        if (rc) return rc;
        for (int k = 0; k < SPR_STAGE_COUNT_; ++k) ms[k] += rp->stage_ms[k];
    }
    if (c.stop_after >= 0 && c.stop_after < SPR_STAGE_IMAGE) return SPR_OK;
    const SrgbTables st = build_srgb_tables();
    rp->image.assign((size_t)W * H * 4, 0);
    const double scale = 1.0 / (68719476736.0 * 256.0);
    for (size_t i = 0; i < (size_t)W * H; ++i) {
        const int64_t *q = sums.data() + 4 * i;
        const float ar = (float)((double)q[0] * scale), ag = (float)((double)q[1] * scale);
        const float ab = (float)((double)q[2] * scale), aa = (float)((double)q[3] * scale);
        uint8_t *o = rp->image.data() + 4 * i;
        if (c.srgb) {
            o[0] = (uint8_t)enc_srgb(st, ar);
            o[1] = (uint8_t)enc_srgb(st, ag);
            o[2] = (uint8_t)enc_srgb(st, ab);
        } else {
            o[0] = (uint8_t)enc_lin(ar);
            o[1] = (uint8_t)enc_lin(ag);
            o[2] = (uint8_t)enc_lin(ab);
        }
        o[3] = (uint8_t)enc_lin(aa);
    }
    std::memcpy(rp->stage_ms, ms, sizeof(ms));
    return SPR_OK;
}

extern "C" int orc_get(const orc_result *r, int32_t stage, const void **ptr, size_t *bytes) {
    if (!r || !ptr || !bytes) return SPR_ERR_INVALID_ARG;
    switch (stage) {
    case SPR_STAGE_TVERTEX: *ptr = r->tvertex.data(); *bytes = r->tvertex.size() * sizeof(F2); break;
    case SPR_STAGE_PATH_VISIBLE: *ptr = r->path_visible.data(); *bytes = r->path_visible.size(); break;
    case SPR_STAGE_CURVE_COUNT: *ptr = r->curve_count.data(); *bytes = r->curve_count.size() * 4; break;
    case SPR_STAGE_INTERSECTION: *ptr = r->entries.data(); *bytes = r->entries.size() * 8; break;
    case SPR_STAGE_FRAG_KEY: *ptr = r->key.data(); *bytes = r->key.size() * 4; break;
    case SPR_STAGE_FRAG_PID: *ptr = r->pid.data(); *bytes = r->pid.size() * 4; break;
    case SPR_STAGE_FRAG_WN: *ptr = r->wn.data(); *bytes = r->wn.size(); break;
    case SPR_STAGE_FRAG_MASK: *ptr = r->mask.data(); *bytes = r->mask.size() * 4; break;
    case SPR_STAGE_SORT_PERM: *ptr = r->perm.data(); *bytes = r->perm.size() * 4; break;
    case SPR_STAGE_SORT_KEY: *ptr = r->skey.data(); *bytes = r->skey.size() * 4; break;
    case SPR_STAGE_WN_SCAN: *ptr = r->wn_scan.data(); *bytes = r->wn_scan.size(); break;
    case SPR_STAGE_MERGED_MASK: *ptr = r->merged_mask.data(); *bytes = r->merged_mask.size() * 4; break;
    case SPR_STAGE_DRAW_LIST: *ptr = r->draw.data(); *bytes = r->draw.size() * 16; break;
    case SPR_STAGE_IMAGE: *ptr = r->image.data(); *bytes = r->image.size(); break;
    default: return SPR_ERR_INVALID_ARG;
    }
    return SPR_OK;
}

extern "C" int orc_counts(const orc_result *r, spr_element_number *out) {
    if (!r || !out) return SPR_ERR_INVALID_ARG;
    *out = r->counts;
    return SPR_OK;
}

extern "C" int orc_stage_ms(const orc_result *r, double *ms, int32_t capacity) {
    if (!r || !ms) return SPR_ERR_INVALID_ARG;
    for (int i = 0; i < capacity && i < SPR_STAGE_COUNT_; ++i) ms[i] = r->stage_ms[i];
    return SPR_OK;
}

extern "C" void orc_free(orc_result *r) { delete r; }

extern "C" int orc_sample_positions(int32_t samples, float *out) {
    if ((samples != 8 && samples != 16 && samples != 32 && samples != 256) || !out) return SPR_ERR_INVALID_ARG;
    std::vector<F2> c = cell_samples(samples);
    std::memcpy(out, c.data(), c.size() * sizeof(F2));
    return SPR_OK;
}

extern "C" int orc_pass_samples_256(int32_t pass, float *out) {
    if (pass < 0 || pass >= 8 || !out) return SPR_ERR_INVALID_ARG;
    std::vector<F2> p = pass_samples_256(pass);
    std::memcpy(out, p.data(), p.size() * sizeof(F2));
    return SPR_OK;
}

extern "C" int orc_pass_mask_table_256(int32_t pass, uint32_t *out) {
    if (pass < 0 || pass >= 8 || !out) return SPR_ERR_INVALID_ARG;
    std::vector<uint32_t> t = build_pass_mask_table_256(pass);
    std::memcpy(out, t.data(), t.size() * 4);
    return SPR_OK;
}

extern "C" int orc_mask_table(int32_t samples, uint32_t *out) {
    if ((samples != 8 && samples != 16 && samples != 32) || !out) return SPR_ERR_INVALID_ARG;
    std::vector<uint32_t> t = build_mask_table(samples);
    std::memcpy(out, t.data(), t.size() * 4);
    return SPR_OK;
}

extern "C" int orc_srgb_tables(float *decode256, float *thresholds255, uint8_t *bins4096) {
    SrgbTables t = build_srgb_tables();
    if (decode256) std::memcpy(decode256, t.decode, sizeof(t.decode));
    if (thresholds255) std::memcpy(thresholds255, t.threshold, sizeof(t.threshold));
    if (bins4096) std::memcpy(bins4096, t.bin, sizeof(t.bin));
    return SPR_OK;
}

extern "C" int orc_fetch_pixel_table(int32_t samples, float p0x, float p0y, float p1x, float p1y,
                                     uint32_t *out_words) {
    if ((samples != 8 && samples != 16 && samples != 32) || !out_words) return SPR_ERR_INVALID_ARG;
    static std::vector<uint32_t> t8, t16, t32;
    std::vector<uint32_t> &t = samples == 8 ? t8 : (samples == 16 ? t16 : t32);
    if (t.empty()) t = build_mask_table(samples);
    fetch_pixel_table(t.data(), samples / 8, F2{p0x, p0y}, F2{p1x, p1y}, out_words);
    return SPR_OK;
}

// testFetchTable_8 / _32 (ras_qm_mask.h:601-713, disabled in the reference):
// every segment between two points of a res x res lattice of the unit cell
// (P0.y != P1.y), table fetch against the exact "sample right of segment"
// test; hist[k] counts segments whose worst pixel word differs in k bits.
extern "C" int orc_fetch_table_selftest(int32_t samples, int32_t res, int64_t *hist33) {
    if ((samples != 8 && samples != 16 && samples != 32) || res < 2 || !hist33) return SPR_ERR_INVALID_ARG;
    std::vector<uint32_t> t = build_mask_table(samples);
    std::vector<F2> cs = cell_samples(samples);
    const int words = samples / 8;
    for (int i = 0; i < 33; ++i) hist33[i] = 0;
    const float step = 1.f / (res - 1.f);
    for (int p1 = 0; p1 < res * res; ++p1)
        for (int p0 = 0; p0 < res * res; ++p0) {
            const int y0 = p0 / res, x0 = p0 - y0 * res, y1 = p1 / res, x1 = p1 - y1 * res;
            if (y0 == y1) continue;
            F2 P0{step * (float)x0, step * (float)y0}, P1{step * (float)x1, step * (float)y1};
            uint32_t got[4];
            fetch_pixel_table(t.data(), words, P0, P1, got);
            int worst = 0;
            if (samples == 8) {
                uint32_t acc = 0;
                for (int j = 0; j < 4; ++j) {
                    uint32_t d = 0;
                    for (int k = 0; k < 8; ++k) {
                        F2 P = cs[j * 8 + k];
                        if (P.x > (P.y - P0.y) / (P1.y - P0.y) * (P1.x - P0.x) + P0.x) d |= 1u << k;
                    }
                    acc |= d << (8 * j);
                }
                worst = __builtin_popcount(got[0] ^ acc);
            } else {
                for (int j = 0; j < words; ++j) {
                    uint32_t d = 0;
                    for (int k = 0; k < 32; ++k) {
                        F2 P = cs[j * 32 + k];
                        if (P.x > (P.y - P0.y) / (P1.y - P0.y) * (P1.x - P0.x) + P0.x) d |= 1u << k;
                    }
                    worst = std::max(worst, __builtin_popcount(got[j] ^ d));
                }
            }
            hist33[worst]++;
        }
    return SPR_OK;
}

extern "C" int orc_vertical_mask(int32_t samples, float y, uint32_t *out_words) {
    if ((samples != 8 && samples != 16 && samples != 32) || !out_words) return SPR_ERR_INVALID_ARG;
    uint32_t tmp[4];
    vertical_mask(samples, y, tmp);
    std::memcpy(out_words, tmp, 4 * (samples / 8));
    return SPR_OK;
}

extern "C" int orc_vertical_mask2(int32_t samples, float y0, float y1, uint32_t *out_words) {
    if ((samples != 8 && samples != 16 && samples != 32) || !out_words) return SPR_ERR_INVALID_ARG;
    uint32_t tmp[4];
    vertical_mask2(samples, y0, y1, tmp);
    std::memcpy(out_words, tmp, 4 * (samples / 8));
    return SPR_OK;
}

// ====================================================== differentiable ==
// Reference of the differentiable render (float composite + edge-sampled
// adjoint) of the library, restated per pixel and sample.  Colours and
// gradients are accumulated in double; the geometric decisions (which sample
// row a chord crosses, the crossing's pixel, the winding on either side) use
// the same float arithmetic as the device so both sides take the same
// crossings.
namespace {

struct Basis {
    double B[4];
    double dx, dy;
};

Basis curve_basis_d(int type, float w, const double *px, const double *py, double t) {
    Basis b{{0, 0, 0, 0}, 0, 0};
    const double u = 1.0 - t;
    if (type == kLinear) {
        b.B[0] = u;
        b.B[1] = t;
        b.dx = px[1] - px[0];
        b.dy = py[1] - py[0];
    } else if (type == kQuad) {
        b.B[0] = u * u;
        b.B[1] = 2 * t * u;
        b.B[2] = t * t;
        b.dx = 2 * (u * (px[1] - px[0]) + t * (px[2] - px[1]));
        b.dy = 2 * (u * (py[1] - py[0]) + t * (py[2] - py[1]));
    } else if (type == kCubic) {
        b.B[0] = u * u * u;
        b.B[1] = 3 * t * u * u;
        b.B[2] = 3 * t * t * u;
        b.B[3] = t * t * t;
        b.dx = 3 * (u * u * (px[1] - px[0]) + 2 * t * u * (px[2] - px[1]) + t * t * (px[3] - px[2]));
        b.dy = 3 * (u * u * (py[1] - py[0]) + 2 * t * u * (py[2] - py[1]) + t * t * (py[3] - py[2]));
    } else {
        const double b0 = u * u, b1 = 2 * t * u * w, b2 = t * t, Wt = b0 + b1 + b2;
        const double iW = Wt != 0 ? 1.0 / Wt : 0.0;
        b.B[0] = b0 * iW;
        b.B[1] = b1 * iW;
        b.B[2] = b2 * iW;
        const double nx = b0 * px[0] + b1 * px[1] + b2 * px[2], ny = b0 * py[0] + b1 * py[1] + b2 * py[2];
        const double dnx = 2 * (u * (w * px[1] - px[0]) + t * (px[2] - w * px[1]));
        const double dny = 2 * (u * (w * py[1] - py[0]) + t * (py[2] - w * py[1]));
        const double dW = 2 * (u * (w - 1.0) + t * (1.0 - w));
        b.dx = (dnx - nx * iW * dW) * iW;
        b.dy = (dny - ny * iW * dW) * iW;
    }
    return b;
}

// dC/dP_j for a chord end: (dCx/dPx, dCx/dPy, dCy/dPx, dCy/dPy) per j.
void end_jacobian_d(int type, float w, const double *px, const double *py, double t, uint32_t flags, bool fixed,
                    double (*dC)[4]) {
    const Basis b = curve_basis_d(type, w, px, py, t);
    int kind = 0;
    if (!fixed && !(flags & 2u)) kind = (flags & 1u) ? 2 : 1;
    if (kind == 1 && std::fabs(b.dx) < 1e-12) kind = 0;
    if (kind == 2 && std::fabs(b.dy) < 1e-12) kind = 0;
    for (int j = 0; j < 4; ++j) {
        const double B = b.B[j];
        dC[j][0] = dC[j][1] = dC[j][2] = dC[j][3] = 0.0;
        if (kind == 0) {
            dC[j][0] = B;
            dC[j][3] = B;
        } else if (kind == 1) {
            dC[j][2] = -(b.dy / b.dx) * B;
            dC[j][3] = B;
        } else {
            dC[j][0] = B;
            dC[j][1] = -(b.dx / b.dy) * B;
        }
    }
}

inline uint32_t row_bit(const uint32_t *m, int S, int px, int r) {
    if (S == 32) return (m[2 * px + (r >> 5)] >> (r & 31)) & 1u;
    if (S == 16) return (m[px] >> r) & 1u;
    return (m[0] >> r) & 1u;
}

inline bool filled_w(int w, int rule) { return rule == 0 ? (w & 0x7f) != 0 : (w & 1) != 0; }

}  // namespace

extern "C" int orc_diff(const spr_scene_view *scene, const orc_config *cfgp, const float *fill,
                        const float *grad_image, double *image, double *grad_fill, double *grad_vertex,
                        double *grad_affine) {
    if (!scene || !cfgp || !fill || !image) return SPR_ERR_INVALID_ARG;
    if (grad_image && (!grad_fill || !grad_vertex)) return SPR_ERR_INVALID_ARG;
    if (grad_affine && !scene->path_affine) return SPR_ERR_INVALID_ARG;
    orc_config cfg = *cfgp;
    cfg.stop_after = SPR_STAGE_DRAW_LIST;
    // 256 samples: 8 passes of 32 (their samples and shifts), each pixel the
    // mean over all passes' samples
    const int passes = cfg.samples == 256 ? 8 : 1;
    if (passes > 1) cfg.samples = 32;
    const int W = cfg.width, H = cfg.height, S = cfg.samples, WORDS = S / 8;
    const int Sd = S * passes;
    const uint32_t P = scene->n_paths, V = scene->n_vertices;
    std::fill(image, image + 4 * (size_t)W * H, 0.0);
    std::vector<double> gt;
    if (grad_image) {
        std::fill(grad_fill, grad_fill + 4 * (size_t)P, 0.0);
        gt.assign(2 * (size_t)V, 0.0);
    }
    std::unique_ptr<orc_result> hold(new orc_result());
    for (int pass = 0; pass < passes; ++pass) {
    *hold = orc_result();
    const int rc = run_frame(scene, cfg, passes > 1 ? pass : -1, *hold, nullptr);
    if (rc) return rc;
    const orc_result &r = *hold;
    const int64_t nf = (int64_t)r.entries.size();
    // items touching each pixel, in draw order
    std::vector<std::vector<int32_t>> items((size_t)W * H);
    for (size_t it = 0; it < r.draw.size(); ++it) {
        const Int4 d = r.draw[it];
        const int x = (int)((uint32_t)d.x & 0xFFFFu), y = (int)(int16_t)(uint16_t)((uint32_t)d.x >> 16);
        const int len = d.w != 0 ? 2 : d.y;
        for (int Y = y; Y < y + 2; ++Y)
            for (int X = x; X < x + len; ++X)
                if (X >= 0 && X < W && Y >= 0 && Y < H) items[(size_t)Y * W + X].push_back((int32_t)it);
    }
    struct Tape {
        int32_t it;
        double c[4];
        bool cov;
    };
    std::vector<Tape> tape;
    for (int Y = 0; Y < H; ++Y)
        for (int X = 0; X < W; ++X) {
            const std::vector<int32_t> &lst = items[(size_t)Y * W + X];
            const int pxc = X & 1, pyc = Y & 1, k4 = pxc * 2 + pyc;
            double G[4] = {0, 0, 0, 0};
            if (grad_image)
                for (int c = 0; c < 4; ++c) G[c] = grad_image[4 * ((size_t)Y * W + X) + c] / Sd;
            for (int i = 0; i < S; ++i) {
                double col[4] = {1, 1, 1, 1};
                tape.clear();
                for (int32_t it : lst) {
                    const Int4 d = r.draw[it];
                    bool cov = true;
                    if (d.w != 0) {
                        const uint32_t *mm = r.merged_mask.data() + (size_t)(d.w - 1) * WORDS;
                        uint32_t bit;
                        if (S == 8) bit = (mm[0] >> (8 * k4 + i)) & 1u;
                        else if (S == 16) bit = (mm[k4 >> 1] >> (16 * (k4 & 1) + i)) & 1u;
                        else bit = (mm[k4] >> i) & 1u;
                        cov = bit != 0;
                    }
                    Tape t{it, {col[0], col[1], col[2], col[3]}, cov};
                    tape.push_back(t);
                    if (cov) {
                        const float *f = fill + 4 * (size_t)r.item_path[it];
                        const double a = f[3], om = 1.0 - a;
                        for (int c = 0; c < 3; ++c) col[c] = f[c] * a + col[c] * om;
                        col[3] = a * a + col[3] * om;
                    }
                }
                for (int c = 0; c < 4; ++c) image[4 * ((size_t)Y * W + X) + c] += col[c] / Sd;
                if (!grad_image) continue;
                double lam[4] = {G[0], G[1], G[2], G[3]};
                const int rrow = pyc * S + i;
                const float yr = ((float)rrow + 0.5f) / (float)(2 * S);
                for (int e = (int)tape.size() - 1; e >= 0; --e) {
                    const Tape &t = tape[e];
                    const Int4 d = r.draw[t.it];
                    const uint32_t path = r.item_path[t.it];
                    const float *f = fill + 4 * (size_t)path;
                    const double a = f[3], om = 1.0 - a;
                    const double *cb = t.c;
                    const double J = lam[0] * a * (f[0] - cb[0]) + lam[1] * a * (f[1] - cb[1]) +
                                     lam[2] * a * (f[2] - cb[2]) + lam[3] * a * (a - cb[3]);
                    if (t.cov) {
                        double *gf = grad_fill + 4 * (size_t)path;
                        for (int c = 0; c < 3; ++c) gf[c] += lam[c] * a;
                        gf[3] += lam[0] * (f[0] - cb[0]) + lam[1] * (f[1] - cb[1]) + lam[2] * (f[2] - cb[2]) +
                                 lam[3] * (2 * a - cb[3]);
                        for (int c = 0; c < 4; ++c) lam[c] *= om;
                    }
                    if (d.w == 0 || J == 0.0) continue;
                    // crossings of the path's chords in this cell with sample row rrow
                    const int64_t h = r.heads[d.w - 1];
                    const int32_t kh = r.skey[h];
                    const uint32_t ph = r.pid[h] & 0x3FFFFFFFu;
                    const int w0 = r.wn_scan[h];
                    const int rule = scene->path_fill_rule[path];
                    auto in_group = [&](int64_t j) {
                        return j < nf && r.skey[j] == kh && (r.pid[j] & 0x3FFFFFFFu) == ph;
                    };
                    for (int64_t j = h; in_group(j); ++j) {
                        const int32_t raw = r.perm[j];
                        const int chg = (int32_t)r.pid[raw] >> 30;
                        if (chg == 0) continue;
                        const float *q = r.chord.data() + 4 * (size_t)raw;
                        if (q[1] == q[3]) continue;
                        uint32_t vm[4];
                        vertical_mask2(S, q[1], q[3], vm);
                        if (!row_bit(vm, S, pxc, rrow)) continue;
                        const float slope = (q[2] - q[0]) / (q[3] - q[1]);
                        const float lamf = (yr - q[1]) / (q[3] - q[1]);
                        const float xc = q[0] + (yr - q[1]) * slope;
                        const int pc = std::min(std::max((int)std::floor(xc * 2.f), 0), 1);
                        if (pc != pxc) continue;
                        int Wn = w0;
                        for (int64_t j2 = h; in_group(j2); ++j2) {
                            const int32_t raw2 = r.perm[j2];
                            const int chg2 = (int32_t)r.pid[raw2] >> 30;
                            if (chg2 == 0) continue;
                            uint32_t bit = 0;
                            if (j2 != j) {
                                const float *q2 = r.chord.data() + 4 * (size_t)raw2;
                                if (q2[1] != q2[3]) {
                                    uint32_t vm2[4];
                                    vertical_mask2(S, q2[1], q2[3], vm2);
                                    if (row_bit(vm2, S, pxc, rrow)) {
                                        const float x2 = q2[0] + (yr - q2[1]) * ((q2[2] - q2[0]) / (q2[3] - q2[1]));
                                        bit = xc > x2 ? 1u : 0u;
                                    }
                                }
                            }
                            bit ^= row_bit(r.lmask.data() + (size_t)raw2 * WORDS, S, pxc, rrow);
                            Wn += chg2 * (int)bit;
                        }
                        const bool cl = filled_w(Wn, rule), cr = filled_w(Wn + chg, rule);
                        if (cl == cr) continue;
                        const double dLdx = cl ? J : -J;
                        const Int2 e0 = r.entries[raw];
                        const Int2 e1 = raw + 1 < nf ? r.entries[raw + 1] : Int2{-1, 0x3f800000};
                        float t0 = float_of((uint32_t)e0.y & 0xFFFFFFFCu), t1 = float_of((uint32_t)e1.y & 0xFFFFFFFCu);
                        if (t0 < 0) t0 = 0.f;
                        if (t1 < 0) t1 = 0.f;
                        const bool end1 = e0.x != e1.x;
                        if (end1) t1 = 1.f;
                        const int cid = e0.x;
                        const int type = scene->curve_type[cid];
                        const float wgt = type == kRational ? scene->curve_arc_w[cid] : 0.f;
                        const uint32_t vp = scene->curve_vertex_pos[cid];
                        const int n = type & 7;
                        double px[4] = {0, 0, 0, 0}, py[4] = {0, 0, 0, 0};
                        for (int k = 0; k < n; ++k) {
                            px[k] = r.tvertex[vp + k].x;
                            py[k] = r.tvertex[vp + k].y;
                        }
                        double dC0[4][4], dC1[4][4];
                        end_jacobian_d(type, wgt, px, py, t0, (uint32_t)e0.y & 3u, t0 == 0.f || t0 == 1.f, dC0);
                        end_jacobian_d(type, wgt, px, py, t1, end1 ? 0u : ((uint32_t)e1.y & 3u),
                                       end1 || t1 == 0.f || t1 == 1.f, dC1);
                        const double l = lamf, sl = slope;
                        for (int k = 0; k < n; ++k) {
                            const double gx = (1 - l) * dC0[k][0] + l * dC1[k][0] - sl * ((1 - l) * dC0[k][2] + l * dC1[k][2]);
                            const double gy = (1 - l) * dC0[k][1] + l * dC1[k][1] - sl * ((1 - l) * dC0[k][3] + l * dC1[k][3]);
                            gt[2 * (vp + k)] += dLdx * gx;
                            gt[2 * (vp + k) + 1] += dLdx * gy;
                        }
                    }
                }
            }
        }
    }  // passes
    const orc_result &r = *hold;
    if (!grad_image) return SPR_OK;
    // transformed vertex -> input vertex and path affine
    float m[16];
    for (int k = 0; k < 16; ++k) m[k] = cfg.has_transform ? cfg.transform[k] : ((k % 5 == 0) ? 1.f : 0.f);
    if (grad_affine) std::fill(grad_affine, grad_affine + 6 * (size_t)P, 0.0);
    std::vector<uint32_t> vmap(V);
    for (uint32_t i = 0; i < V; ++i) vmap[i] = i;
    for (uint32_t c = 0; c < scene->n_curves; ++c)
        if (r.reversed[c]) {
            const uint32_t p0 = scene->curve_vertex_pos[c];
            const int vn = scene->curve_type[c] & 7;
            for (int k = 0; k < vn; ++k) vmap[p0 + k] = p0 + vn - 1 - k;
        }
    for (uint32_t i = 0; i < V; ++i) {
        // the stored (unified) vertex i holds the input vertex vmap[i]
        const double vx = scene->vertex[2 * vmap[i]], vy = scene->vertex[2 * vmap[i] + 1];
        const uint32_t pid = scene->vertex_path_id[vmap[i]];
        double A[6] = {1, 0, 0, 1, 0, 0};
        double xa = vx, ya = vy;
        if (scene->path_affine) {
            for (int k = 0; k < 6; ++k) A[k] = scene->path_affine[6 * (size_t)pid + k];
            xa = A[0] * vx + A[2] * vy + A[4];
            ya = A[1] * vx + A[3] * vy + A[5];
        }
        double ov[4], dox[4], doy[4];
        for (int rr = 0; rr < 4; ++rr) {
            ov[rr] = m[4 * rr] * xa + m[4 * rr + 1] * ya + m[4 * rr + 3];
            dox[rr] = m[4 * rr];
            doy[rr] = m[4 * rr + 1];
        }
        double q[3], qx[3], qy[3];
        for (int rr = 0; rr < 3; ++rr) {
            q[rr] = ov[rr] / ov[3];
            qx[rr] = (dox[rr] - q[rr] * dox[3]) / ov[3];
            qy[rr] = (doy[rr] - q[rr] * doy[3]) / ov[3];
        }
        const double w = W, hh = H, z = std::min(W, H), cutoff = -z * 0.5;
        if (q[2] < cutoff) {
            q[2] = cutoff;
            qx[2] = qy[2] = 0;
        }
        const double den = q[2] + z, f = z / den, fx = -f / den * qx[2], fy = -f / den * qy[2];
        const double Jxx = qx[0] * f + (q[0] - w * .5) * fx, Jxy = qy[0] * f + (q[0] - w * .5) * fy;
        const double Jyx = qx[1] * f + (q[1] - hh * .5) * fx, Jyy = qy[1] * f + (q[1] - hh * .5) * fy;
        const double gx = gt[2 * i], gy = gt[2 * i + 1];
        const double gxa = Jxx * gx + Jyx * gy, gya = Jxy * gx + Jyy * gy;
        grad_vertex[2 * vmap[i]] = A[0] * gxa + A[1] * gya;
        grad_vertex[2 * vmap[i] + 1] = A[2] * gxa + A[3] * gya;
        if (grad_affine) {
            double *Ga = grad_affine + 6 * (size_t)pid;
            Ga[0] += gxa * vx;
            Ga[1] += gya * vx;
            Ga[2] += gxa * vy;
            Ga[3] += gya * vy;
            Ga[4] += gxa;
            Ga[5] += gya;
        }
    }
    return SPR_OK;
}

// ------------------------------------ FP64 check of the crossing points --
// For the benchmark's accuracy report: how far the FP32 crossing points of
// the intersection entries (k_make_intersection_impl_1, ras_cut.h:837-1241,
// as emitted above) lie from the exact crossings of the same curves with the
// same cut lines.  The curves are the FP32 transformed vertices; the exact
// crossing t* solves P_side(t) = c in double on the entry's monotone piece
// (60 bisection steps, then Newton polish), and the error is measured along
// the cut line: for a crossing of a horizontal line y = c the x error, for a
// vertical line x = c the y error, of the point the fragment stage uses (the
// FP32 curve_coord at the entry's t, flag bits cleared).
namespace {

double coord_d(int type, double w, const float *v, double t) {
    const double a = v[0], b = v[1], c = v[2], d = v[3], u = 1.0 - t;
    switch (type) {
    case kLinear: return a * u + b * t;
    case kQuad: return a * u * u + 2.0 * b * u * t + c * t * t;
    case kCubic: return a * u * u * u + 3.0 * b * u * u * t + 3.0 * c * u * t * t + d * t * t * t;
    default: {  // rational quadratic with weights (1, w, 1); v[1] is the raw middle coordinate
        const double num = a * u * u + 2.0 * w * b * u * t + c * t * t;
        const double den = u * u + 2.0 * w * u * t + t * t;
        return den != 0.0 ? num / den : 0.0;
    }
    }
}

struct CrossingMeta {
    float t;      // entry t, flag bits cleared
    float t0, t1; // the monotone piece (flag bits cleared)
    float c;      // cut-line coordinate
    int side;     // 0: vertical line x = c, 1: horizontal line y = c
    bool crossing;
};

// emit_curve's walk, recording which solve produced each entry.
int emit_meta(const CurveGeom &g, int W, int H, std::vector<CrossingMeta> &out) {
    float t0_ms = 0.f;
    F2 v0{g.px[0], g.py[0]};
    for (int ms = 0; ms < g.n_pieces; ++ms) {
        float traw = g.tcut[ms];
        F2 v1{curve_coord(g.type, g.w, g.px, traw), curve_coord(g.type, g.w, g.py, traw)};
        uint32_t tb = bits_of(traw) & 0xFFFFFFFCu;
        float t1_ms = (std::floor(v1.x) == v1.x) ? float_of(tb | 2u) : float_of(tb | 3u);
        CutRange cr = cut_range(v0, v1, W, H);
        int nx = cr.nx, ny = cr.ny;
        const int n_loop = nx + ny + 1;
        float x = (float)(cr.dx < 0.f ? cr.xe : cr.xb);
        float y = (float)(cr.dy < 0.f ? cr.ye : cr.yb);
        float slot[2] = {t0_ms, t0_ms};
        float slot_c[2] = {0.f, 0.f};
        bool slot_x[2] = {false, false};
        const float p0 = float_of(bits_of(t0_ms) & 0xFFFFFFFCu), p1 = float_of(bits_of(t1_ms) & 0xFFFFFFFCu);
        for (int i = -1; i < n_loop; ++i) {
            float t_solve = 0.f, c = 0.f, t_min;
            int side = 0, took = 0;
            float ntx = slot[0], nty = slot[1];
            if (i == -1) {
                t_min = ntx;
                if (nx == 0) {
                    t_solve = 2.f;
                } else if (ny == 0) {
                    side = 1;
                    t_solve = 2.f;
                } else {
                    nx--;
                    c = x;
                    x += cr.dx;
                }
            } else if (ntx <= nty) {
                t_min = ntx;
                took = 0;
                if (nx > 0) {
                    nx--;
                    c = x;
                    x += cr.dx;
                } else {
                    t_solve = 2.f;
                }
            } else {
                t_min = nty;
                took = 1;
                side = 1;
                if (ny > 0) {
                    ny--;
                    c = y;
                    y += cr.dy;
                } else {
                    t_solve = 2.f;
                }
            }
            if (i >= 0) {
                out.push_back({float_of(bits_of(t_min) & 0xFFFFFFFCu), p0, p1, slot_c[took], took, slot_x[took]});
            }
            const bool solved = t_solve < 2.f;
            if (solved) t_solve = solve_crossing(g, side ? g.py : g.px, c, t_min, t1_ms);
            slot[side] = float_of((bits_of(t_solve) & 0xFFFFFFFCu) | (uint32_t)side);
            slot_c[side] = c;
            slot_x[side] = solved;
        }
        t0_ms = t1_ms;
        v0 = v1;
    }
    return (int)out.size();
}

// Exact root of P(t) = c on [a, b] in double; false without a sign change.
bool root_d(int type, double w, const float *P, double c, double a, double b, double *t_out) {
    double fa = coord_d(type, w, P, a) - c, fb = coord_d(type, w, P, b) - c;
    if (fa == 0.0) return *t_out = a, true;
    if (fb == 0.0) return *t_out = b, true;
    if ((fa < 0.0) == (fb < 0.0)) return false;
    for (int it = 0; it < 60; ++it) {
        const double m = 0.5 * (a + b), fm = coord_d(type, w, P, m) - c;
        if (fm == 0.0) return *t_out = m, true;
        if ((fm < 0.0) == (fa < 0.0)) a = m, fa = fm;
        else b = m, fb = fm;
    }
    *t_out = std::fabs(fa) < std::fabs(fb) ? a : b;
    return true;
}

}  // namespace

extern "C" int orc_intersection_error(const spr_scene_view *scene, const float *tvertex, const int32_t *entries,
                                      int64_t n_entries, int32_t width, int32_t height, int32_t threads,
                                      orc_xerr *out) {
    if (!scene || !out || (n_entries > 0 && (!tvertex || !entries))) return SPR_ERR_INVALID_ARG;
    *out = orc_xerr{};
    out->worst_entry = -1;
    const uint32_t C = scene->n_curves;
    // entries of curve i start at offs[i] (they are grouped by curve id)
    std::vector<int64_t> offs(C + 1, n_entries);
    {
        int64_t j = 0;
        for (uint32_t i = 0; i <= C; ++i) {
            while (j < n_entries && (uint32_t)entries[2 * j] < i) ++j;
            offs[i] = j;
        }
    }
    const int nthreads = threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
    struct Acc {
        double max_err = 0, sum_err = 0, max_resid = 0;
        int64_t n = 0, mismatched = 0, unbracketed = 0, over_1px = 0, worst = -1;
    };
    std::vector<Acc> acc(nthreads);
    std::atomic<int64_t> next{0};
    auto work = [&](int tid) {
        Acc &A = acc[tid];
        std::vector<CrossingMeta> meta;
        for (;;) {
            const int64_t c0 = next.fetch_add(256);
            if (c0 >= C) break;
            for (int64_t i = c0; i < std::min<int64_t>(C, c0 + 256); ++i) {
                CurveGeom g;
                g.type = scene->curve_type[i];
                g.w = (g.type == kRational) ? scene->curve_arc_w[i] : 0.f;
                const uint32_t p = scene->curve_vertex_pos[i];
                const int nv = g.type & 7;
                for (int k = 0; k < 4; ++k) {
                    g.px[k] = k < nv ? tvertex[2 * ((size_t)p + k)] : 0.f;
                    g.py[k] = k < nv ? tvertex[2 * ((size_t)p + k) + 1] : 0.f;
                }
                const int64_t b = offs[i], e = offs[i + 1];
                if (b == e) continue;
                monotonize(g, true);
                meta.clear();
                emit_meta(g, width, height, meta);
                if ((int64_t)meta.size() != e - b) {
                    A.mismatched += e - b;
                    continue;
                }
                for (int64_t k = b; k < e; ++k) {
                    const CrossingMeta &m = meta[k - b];
                    const float t = float_of((uint32_t)entries[2 * k + 1] & 0xFFFFFFFCu);
                    if (bits_of(t) != bits_of(m.t)) {
                        ++A.mismatched;
                        continue;
                    }
                    if (!m.crossing) continue;
                    const float *P = m.side ? g.py : g.px;  // the coordinate fixed by the cut line
                    const float *Q = m.side ? g.px : g.py;  // the coordinate along it
                    double ts;
                    if (!root_d(g.type, g.w, P, m.c, m.t0, m.t1, &ts)) {
                        ++A.unbracketed;
                        continue;
                    }
                    const double q_exact = coord_d(g.type, g.w, Q, ts);
                    const double q_used = curve_coord(g.type, g.w, Q, t);
                    const double err = std::fabs(q_used - q_exact);
                    const double resid = std::fabs((double)curve_coord(g.type, g.w, P, t) - m.c);
                    ++A.n;
                    A.sum_err += err;
                    if (err > 1.0) ++A.over_1px;
                    if (err > A.max_err) A.max_err = err, A.worst = k;
                    A.max_resid = std::max(A.max_resid, resid);
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nthreads; ++t) pool.emplace_back(work, t);
    work(0);
    for (auto &t : pool) t.join();
    double sum = 0;
    for (const Acc &A : acc) {
        out->n_crossings += A.n;
        out->n_mismatched += A.mismatched;
        out->n_unbracketed += A.unbracketed;
        out->n_over_1px += A.over_1px;
        sum += A.sum_err;
        if (A.worst >= 0 && (out->worst_entry < 0 || A.max_err > out->max_err_px)) {
            out->max_err_px = A.max_err;
            out->worst_entry = A.worst;
        }
        out->max_resid_px = std::max(out->max_resid_px, A.max_resid);
    }
    out->mean_err_px = out->n_crossings ? sum / (double)out->n_crossings : 0.0;
    return SPR_OK;
}
