// spr_device.cuh -- device-side arithmetic of the scanline pipeline.
//
// Everything here is bit-exact by construction against a host restatement
// compiled with -ffp-contract=off: this translation unit is compiled with
// --fmad=false (no fused multiply-add), IEEE division and square root, and
// the float->int conversions and shifts spell out the CUDA/PTX semantics
// (saturating conversion, NaN -> 0, shift counts >= width give 0).
#pragma once

#include <cstdint>

#include "../../include/spr.h"

namespace spr {

constexpr int kLinear = SPR_CURVE_LINEAR;
constexpr int kQuad = SPR_CURVE_QUADRATIC;
constexpr int kCubic = SPR_CURVE_CUBIC;
constexpr int kRational = SPR_CURVE_RATIONAL;
constexpr int32_t kInvalidKey = (int32_t)0xFFFEFFFEu;

__device__ __forceinline__ uint32_t fbits(float f) { return __float_as_uint(f); }
__device__ __forceinline__ float ffrom(uint32_t u) { return __uint_as_float(u); }
__device__ __forceinline__ int32_t cvt_rmi(float x) { return __float2int_rd(x); }
__device__ __forceinline__ int32_t cvt_rzi(float x) { return __float2int_rz(x); }
__device__ __forceinline__ int32_t cvt_rzi_d(double x) { return __double2int_rz(x); }
__device__ __forceinline__ int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
__device__ __forceinline__ uint32_t shr32(uint32_t v, int32_t s) { return (s < 0 || s >= 32) ? 0u : (v >> s); }
__device__ __forceinline__ uint64_t shr64(uint64_t v, int32_t s) { return (s < 0 || s >= 64) ? 0ull : (v >> s); }

// fmaxf / fminf with a fixed signed-zero rule (+0 for max, -0 for min).
__device__ __forceinline__ float fmax_r(float a, float b) {
    if (isnan(a)) return b;
    if (isnan(b)) return a;
    if (a > b) return a;
    if (b > a) return b;
    return signbit(a) ? b : a;
}
__device__ __forceinline__ float fmin_r(float a, float b) {
    if (isnan(a)) return b;
    if (isnan(b)) return a;
    if (a < b) return a;
    if (b < a) return b;
    return signbit(a) ? a : b;
}

__device__ __forceinline__ float safe_rcp(float a) { return a != 0.f ? (1.f / a) : 0.f; }
__device__ __forceinline__ float lerpf(float a, float b, float t) { return a + t * (b - a); }
__device__ __forceinline__ int32_t floor2(float x) { return (int32_t)((uint32_t)cvt_rmi(x) & 0xFFFFFFFEu); }

// One coordinate of a curve point (de Casteljau; rational quadratics divide
// by the weight polynomial).
__device__ __forceinline__ float curve_coord(int type, float w, const float *v, float t) {
    if (type == kLinear) return lerpf(v[0], v[1], t);
    if (type == kQuad) {
        float a = lerpf(v[0], v[1], t);
        float b = lerpf(v[1], v[2], t);
        return lerpf(a, b, t);
    }
    if (type == kCubic) {
        float q0 = lerpf(v[0], v[1], t);
        float q1 = lerpf(v[1], v[2], t);
        float q2 = lerpf(v[2], v[3], t);
        float l0 = lerpf(q0, q1, t);
        float l1 = lerpf(q1, q2, t);
        return lerpf(l0, l1, t);
    }
    float iv1 = v[1] * w;
    float l0 = lerpf(v[0], iv1, t);
    float l1 = lerpf(iv1, v[2], t);
    float r = lerpf(l0, l1, t);
    float ww = (1 - t) * (1 - t) + 2.f * (1 - t) * t * w + t * t;
    r *= safe_rcp(ww);
    return r;
}

__device__ __forceinline__ float cubic_coord(const float *v, float t) {
    float q0 = lerpf(v[0], v[1], t);
    float q1 = lerpf(v[1], v[2], t);
    float q2 = lerpf(v[2], v[3], t);
    float l0 = lerpf(q0, q1, t);
    float l1 = lerpf(q1, q2, t);
    return lerpf(l0, l1, t);
}

// Roots of a*t^2 + b*t + c in the numerically stable form of the reference.
__device__ __forceinline__ void solve_quad_eq(float a, float b, float c, float *r0, float *r1) {
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
        float SR = sqrtf(R);
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

// Root of the quadratic Bezier coordinate (A, B, C) - D within [t0, t1];
// falls back to t0.
__device__ __forceinline__ float solve_quad_bezier(float iA, float iB, float iC, float iD, float t0, float t1) {
    float a = iA + (-2.f) * iB + iC;
    float b = -2.f * iA + 2.f * iB;
    float c = iA - iD;
    float r0 = 0.f, r1 = 0.f;
    solve_quad_eq(a, b, c, &r0, &r1);
    if (t0 <= r0 && r0 <= t1) return r0;
    if (t0 <= r1 && r1 <= t1) return r1;
    return t0;
}

struct CurveGeom {
    int type;
    float w;
    float px[4], py[4];
};

// Cut lines crossed by the monotone piece v0 -> v1 (clamped to
// [0, (dim & ~1) + 2]).
struct CutRange {
    int xb, xe, yb, ye, nx, ny;
    float dx, dy;
};
__device__ __forceinline__ CutRange cut_range(float v0x, float v0y, float v1x, float v1y, int W, int H) {
    CutRange c;
    if (v0x <= v1x) {
        c.xb = floor2(v0x) + 2;
        c.xe = floor2(v1x);
        c.dx = 2.f;
    } else {
        c.xb = floor2(v1x) + 2;
        c.xe = floor2(v0x);
        c.dx = -2.f;
    }
    if (v0y <= v1y) {
        c.yb = floor2(v0y) + 2;
        c.ye = floor2(v1y);
        c.dy = 2.f;
    } else {
        c.yb = floor2(v1y) + 2;
        c.ye = floor2(v0y);
        c.dy = -2.f;
    }
    const int xmax = (W & ~1) + 2, ymax = (H & ~1) + 2;
    if ((c.xb < 0 && c.xe < 0) || (c.xb > xmax && c.xe > xmax) || (c.xb > c.xe)) {
        c.nx = 0;
    } else {
        c.xb = min(max(c.xb, 0), xmax);
        c.xe = min(max(c.xe, 0), xmax);
        c.nx = max((c.xe - c.xb) / 2 + 1, 0);
    }
    if ((c.yb < 0 && c.ye < 0) || (c.yb > ymax && c.ye > ymax) || (c.yb > c.ye)) {
        c.ny = 0;
    } else {
        c.yb = min(max(c.yb, 0), ymax);
        c.ye = min(max(c.ye, 0), ymax);
        c.ny = max((c.ye - c.yb) / 2 + 1, 0);
    }
    return c;
}

// Monotone cut points (x extrema then y extrema, insertion-sorted) followed
// by t = 1.  Returns the number of monotone pieces (0 when invisible).
__device__ __forceinline__ int monotonize(const CurveGeom &g, bool visible, float *q) {
    int n = 0;
    q[0] = q[1] = q[2] = q[3] = q[4] = 0.f;
    if (!visible) return 0;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        const float *P = c == 0 ? g.px : g.py;
        if (g.type == kQuad) {
            float b = (P[0] - P[1]) + (P[2] - P[1]);
            if (!(fabsf(b) < 1e-6f)) {
                float t = (P[0] - P[1]) / b;
                if (t > 0.f && t < 1.f) q[n++] = t;
            }
        } else if (g.type == kCubic) {
            float r0 = 0.f, r1 = 0.f;
            solve_quad_eq((P[3] - P[0]) + 3.f * (P[1] - P[2]), 2.f * ((P[0] - P[1]) + (P[2] - P[1])), P[1] - P[0],
                          &r0, &r1);
            if (r0 > 0.f && r0 < 1.f) q[n++] = r0;
            if (r1 > 0.f && r1 < 1.f && r1 != r0) q[n++] = r1;
        } else if (g.type == kRational) {
            float w0 = 1.f, w1 = g.w, w2 = 1.f;
            float p0 = w0 * P[0], p1 = w1 * P[1], p2 = w2 * P[2];
            float pw01 = p0 * w1 - p1 * w0;
            float pw12 = p1 * w2 - p2 * w1;
            float pw20 = p2 * w0 - p0 * w2;
            float r0 = 0.f, r1 = 0.f;
            solve_quad_eq(pw01 + pw12 + pw20, -(2.f * pw01 + pw20), pw01, &r0, &r1);
            if (r0 > 0.f && r0 < 1.f) q[n++] = r0;
            if (r1 > 0.f && r1 < 1.f && r1 != r0) q[n++] = r1;
        }
    }
    for (int i = 1; i < n; ++i) {
        float t = q[i];
        int j = i - 1;
        while (j >= 0 && t < q[j]) {
            q[j + 1] = q[j];
            --j;
        }
        q[j + 1] = t;
    }
    q[n++] = 1.f;
    return n;
}

// monotonize() in registers: the same cut points as its insertion sort
// (equal values are interchangeable, so a sorting network gives the same
// array), q[0..n) followed by q[n] = 1, q[k > n] = 0.
__device__ __forceinline__ void cas(float &a, float &b) {
    const float lo = fminf(a, b), hi = fmaxf(a, b);  // (no NaN: candidates lie in (0, 1), unused ones are 2)
    a = lo;
    b = hi;
}
__device__ __forceinline__ int monotonize_r(const CurveGeom &g, bool visible, float (&q)[5]) {
    q[0] = q[1] = q[2] = q[3] = q[4] = 0.f;
    if (!visible) return 0;
    float c[4] = {2.f, 2.f, 2.f, 2.f};  // x roots, then y roots; 2 = none
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float *P = k == 0 ? g.px : g.py;
        float r0 = 2.f, r1 = 2.f;
        if (g.type == kQuad) {
            float b = (P[0] - P[1]) + (P[2] - P[1]);
            if (!(fabsf(b) < 1e-6f)) {
                float t = (P[0] - P[1]) / b;
                if (t > 0.f && t < 1.f) r0 = t;
            }
        } else if (g.type == kCubic || g.type == kRational) {
            float a0 = 0.f, a1 = 0.f;
            if (g.type == kCubic) {
                solve_quad_eq((P[3] - P[0]) + 3.f * (P[1] - P[2]), 2.f * ((P[0] - P[1]) + (P[2] - P[1])), P[1] - P[0],
                              &a0, &a1);
            } else {
                float w0 = 1.f, w1 = g.w, w2 = 1.f;
                float p0 = w0 * P[0], p1 = w1 * P[1], p2 = w2 * P[2];
                float pw01 = p0 * w1 - p1 * w0;
                float pw12 = p1 * w2 - p2 * w1;
                float pw20 = p2 * w0 - p0 * w2;
                solve_quad_eq(pw01 + pw12 + pw20, -(2.f * pw01 + pw20), pw01, &a0, &a1);
            }
            if (a0 > 0.f && a0 < 1.f) r0 = a0;
            if (a1 > 0.f && a1 < 1.f && a1 != a0) r1 = a1;
        }
        c[2 * k] = r0;
        c[2 * k + 1] = r1;
    }
    cas(c[0], c[1]);
    cas(c[2], c[3]);
    cas(c[0], c[2]);
    cas(c[1], c[3]);
    cas(c[1], c[2]);
    const int n = (c[0] < 2.f) + (c[1] < 2.f) + (c[2] < 2.f) + (c[3] < 2.f);
#pragma unroll
    for (int k = 0; k < 4; ++k) q[k] = k < n ? c[k] : (k == n ? 1.f : 0.f);
    q[4] = n == 4 ? 1.f : 0.f;
    return n + 1;
}

// Crossing of coordinate P(t) = c on [tmin, tmax].
__device__ __forceinline__ float solve_crossing(const CurveGeom &g, const float *P, float c, float tmin, float tmax) {
    if (g.type == kLinear) {
        float t = (c - P[0]) * safe_rcp(P[1] - P[0]);
        t = t > tmin ? t : tmin;
        return t < tmax ? t : tmax;
    }
    if (g.type == kQuad) return solve_quad_bezier(P[0], P[1], P[2], c, tmin, tmax);
    if (g.type == kRational) return solve_quad_bezier(P[0] - c, (P[1] - c) * g.w, P[2] - c, 0.f, tmin, tmax);
    float t0 = tmin, t1 = tmax;
    float vt0 = cubic_coord(P, t0);
    float ts = t0;
    if (vt0 != c) {
        float raw_t0 = t0;
        float last = 0.f;
#pragma unroll 4
        for (int it = 0; it < 24; ++it) {
            float tm = (t0 + t1) * .5f;
            float vtm = cubic_coord(P, tm);
            ts = tm;
            last = vtm;
            if ((int32_t)(fbits(vtm - c) ^ fbits(vt0 - c)) >= 0) {
                t0 = tm;
                vt0 = vtm;
            } else {
                t1 = tm;
            }
        }
        if (fabsf(last - c) > 1.f) ts = raw_t0;
    }
    return ts;
}

// Vertical sample-row masks.  Mask bit b of the 2N stacked sample rows of a
// cell column (N = 8: 16 rows, one 32-bit word duplicated for both pixel
// columns; N = 16: 32 rows, words (column 0, column 1); N = 32: 64 rows,
// words (low, high, low, high)).
template <int N>
__device__ __forceinline__ void vertical_mask(float y, uint32_t *out) {
    if (N == 16) {
        int32_t r = cvt_rzi(roundf(y * 32));
        uint32_t m = shr32(0xFFFFFFFFu, wsub(32, r));
        out[0] = m;
        out[1] = m;
    } else if (N == 8) {
        int32_t r = cvt_rzi(roundf(y * 16));
        uint32_t m = shr32(0xffffu, wsub(16, r));
        out[0] = m | (m << 16);
    } else {
        int32_t r = cvt_rzi(roundf(y * 64));
        uint64_t m = shr64(~0ull, wsub(64, r));
        uint32_t m0 = (uint32_t)m, m1 = (uint32_t)(m >> 32);
        out[0] = m0;
        out[1] = m1;
        out[2] = m0;
        out[3] = m1;
    }
}
template <int N>
__device__ __forceinline__ void vertical_mask2(float y0, float y1, uint32_t *out) {
    if (N == 16) {
        int32_t s0 = max(wsub(32, cvt_rzi_d((double)(y0 * 32) + 0.5)), 0);
        int32_t s1 = max(wsub(32, cvt_rzi_d((double)(y1 * 32) + 0.5)), 0);
        uint32_t m = shr32(0xFFFFFFFFu, s0) ^ shr32(0xFFFFFFFFu, s1);
        out[0] = m;
        out[1] = m;
    } else if (N == 8) {
        int32_t s0 = max(wsub(16, cvt_rzi_d((double)(y0 * 16) + 0.5)), 0);
        int32_t s1 = max(wsub(16, cvt_rzi_d((double)(y1 * 16) + 0.5)), 0);
        uint32_t m = shr32(0xffffu, s0) ^ shr32(0xffffu, s1);
        out[0] = m | (m << 16);
    } else {
        int32_t s0 = max(wsub(64, cvt_rzi_d((double)(y0 * 64) + 0.5)), 0);
        int32_t s1 = max(wsub(64, cvt_rzi_d((double)(y1 * 64) + 0.5)), 0);
        uint64_t m = shr64(~0ull, s0) ^ shr64(~0ull, s1);
        uint32_t m0 = (uint32_t)m, m1 = (uint32_t)(m >> 32);
        out[0] = m0;
        out[1] = m1;
        out[2] = m0;
        out[3] = m1;
    }
}

// Texel of the 256x256 half-plane table for the segment P0 -> P1 (cell
// coordinates): the line's normal and offset are folded into a point of the
// unit disk, point-sampled with clamping.
__device__ __forceinline__ int table_texel(float p0x, float p0y, float p1x, float p1y) {
    if (p1y < p0y) {
        float tx = p0x, ty = p0y;
        p0x = p1x;
        p0y = p1y;
        p1x = tx;
        p1y = ty;
    }
    float dx = p1x - p0x, dy = p1y - p0y;
    float vx = dy, vy = -dx;
    float inv = 1.0f / sqrtf(vx * vx + vy * vy);
    float nx = vx * inv, ny = vy * inv;
    float C = nx * p0x + ny * p0y;
    C -= 0.5f * (nx + ny);
    float C_sign = ffrom((fbits(C) & 0x80000000u) + 0x3f800000u);
    float k = fmax_r(1.f - C * C_sign * 0.5f, 0.f) * C_sign;
    float u = (k * nx) * 0.5f + 0.5f;
    float v = (k * ny) * 0.5f + 0.5f;
    int ix = min(max(cvt_rmi(u * 256.f), 0), 255);
    int iy = min(max(cvt_rmi(v * 256.f), 0), 255);
    return iy * 256 + ix;
}

// Cell key (int16 fields offset by 0x7FFF).
__device__ __forceinline__ int key_x(uint32_t k) { return (int16_t)(uint16_t)((k & 0xFFFFu) - 0x7FFFu); }
__device__ __forceinline__ int key_y(uint32_t k) { return (int16_t)(uint16_t)((k >> 16) - 0x7FFFu); }

// Sort key of a cell within its path: the rank of the key as a signed int32
// compressed to (row rank: 12 bits, column: 12 bits).  Rows y >= 2 come
// first (their keys are negative), then the out-of-range sentinel, then
// row 0.
__device__ __forceinline__ uint32_t local_sort_key(int32_t key, int nrows) {
    if (key == kInvalidKey) return (uint32_t)(nrows - 1) << 12;
    int y = key_y((uint32_t)key), x = key_x((uint32_t)key);
    uint32_t rr = y == 0 ? (uint32_t)nrows : (uint32_t)(y / 2 - 1);
    return (rr << 12) | (uint32_t)((x + 2) >> 1);
}
__device__ __forceinline__ int32_t key_from_local(uint32_t lk, int nrows) {
    uint32_t rr = lk >> 12;
    if (rr == (uint32_t)(nrows - 1)) return kInvalidKey;
    int y = rr == (uint32_t)nrows ? 0 : 2 * ((int)rr + 1);
    int x = 2 * (int)(lk & 0xFFFu) - 2;
    return (int32_t)(((uint32_t)(y + 0x7FFF) << 16) | ((uint32_t)(x + 0x7FFF) & 0xFFFFu));
}

}  // namespace spr
