// spr_diff.cu -- differentiable rendering: a float per-sample composite of
// the draw list (forward) and its adjoint (backward).
//
// The coverage pipeline (fragments, sort, winding scan, merged sample masks,
// draw list) is the bit-exact one of spr_kernels.cu.  On top of it every
// sample is composited in linear float RGBA over a white background in
// painter's order, c' = f.rgb * a + c.rgb * (1 - a), c'.a = a * a + c.a *
// (1 - a) (the same blend as the multisample resolve, without the 8-bit
// sRGB storage), and a pixel is the mean of its samples.
//
// Backward, per sample: a tape of the state before every draw item that
// touches the sample's cell is recorded in draw order and swept in reverse
// with the adjoint lambda of the state (lambda *= 1 - a through every
// covering item), giving the exact fill gradients.  Geometry is
// differentiated by edge sampling: a pixel is taken as the mean over its S
// sample rows of the row integral of the composite, so moving the crossing
// x_c of a chord with sample row y_r by dx changes the pixel by
// (c_left - c_right) dx / S.  c_left - c_right is the jump of path k's
// coverage (from the exact winding on both sides of the crossing, the same
// chords, left masks and scanline winding the forward masks use) times
// lambda . (blend_k(c) - c) at the sample of that row.  The crossing moves
// with the chord's end points, which lie on cell lines (x = 2m or y = 2n,
// moving along the line as the curve moves) or at fixed curve parameters
// (curve ends and monotone split points), and so with the curve's control
// points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "spr_device.cuh"
#include "spr_internal.h"

namespace spr {

namespace {

constexpr int kDiffThreads = 512;  // 64 pixels x 8 threads; a thread holds S / 8 samples of one pixel
constexpr int kDiffChunk = 64;     // draw items staged per step
constexpr int kDiffItemAcc = 1024; // items of a bin with shared-memory fill-gradient accumulators
constexpr int kTileW = 32;

__device__ __forceinline__ uint32_t pixel_mask(const uint4 &mm, int S, int k) {
    if (S == 32) return k == 0 ? mm.x : (k == 1 ? mm.y : (k == 2 ? mm.z : mm.w));
    if (S == 16) return ((k < 2 ? mm.x : mm.y) >> (16 * (k & 1))) & 0xFFFFu;
    return (mm.x >> (8 * k)) & 0xFFu;
}

// Bit r of the 2S stacked sample rows of cell column px in a vertical-mask
// word layout (vertical_mask / vertical_mask2).
template <int S>
__device__ __forceinline__ uint32_t row_bit(const uint32_t *m, int px, int r) {
    if constexpr (S == 32) return (m[2 * px + (r >> 5)] >> (r & 31)) & 1u;
    else if constexpr (S == 16) return (m[px] >> r) & 1u;
    else return (m[0] >> r) & 1u;
}

// Curve basis at t: P(t) = sum_j B[j] P_j, and P'(t).
__device__ __forceinline__ void curve_basis(const CurveGeom &g, float t, float *B, float &dx, float &dy) {
    const float u = 1.f - t;
    B[0] = B[1] = B[2] = B[3] = 0.f;
    if (g.type == kLinear) {
        B[0] = u;
        B[1] = t;
        dx = g.px[1] - g.px[0];
        dy = g.py[1] - g.py[0];
    } else if (g.type == kQuad) {
        B[0] = u * u;
        B[1] = 2.f * t * u;
        B[2] = t * t;
        dx = 2.f * (u * (g.px[1] - g.px[0]) + t * (g.px[2] - g.px[1]));
        dy = 2.f * (u * (g.py[1] - g.py[0]) + t * (g.py[2] - g.py[1]));
    } else if (g.type == kCubic) {
        B[0] = u * u * u;
        B[1] = 3.f * t * u * u;
        B[2] = 3.f * t * t * u;
        B[3] = t * t * t;
        dx = 3.f * (u * u * (g.px[1] - g.px[0]) + 2.f * t * u * (g.px[2] - g.px[1]) + t * t * (g.px[3] - g.px[2]));
        dy = 3.f * (u * u * (g.py[1] - g.py[0]) + 2.f * t * u * (g.py[2] - g.py[1]) + t * t * (g.py[3] - g.py[2]));
    } else {  // rational quadratic, weights (1, w, 1)
        const float w = g.w;
        const float b0 = u * u, b1 = 2.f * t * u * w, b2 = t * t;
        const float W = b0 + b1 + b2;
        const float iW = W != 0.f ? 1.f / W : 0.f;
        B[0] = b0 * iW;
        B[1] = b1 * iW;
        B[2] = b2 * iW;
        const float nx = b0 * g.px[0] + b1 * g.px[1] + b2 * g.px[2];
        const float ny = b0 * g.py[0] + b1 * g.py[1] + b2 * g.py[2];
        const float dnx = 2.f * (u * (w * g.px[1] - g.px[0]) + t * (g.px[2] - w * g.px[1]));
        const float dny = 2.f * (u * (w * g.py[1] - g.py[0]) + t * (g.py[2] - w * g.py[1]));
        const float dW = 2.f * (u * (w - 1.f) + t * (1.f - w));
        dx = (dnx - nx * iW * dW) * iW;
        dy = (dny - ny * iW * dW) * iW;
    }
}

// d(end point)/d(control point j) of a chord end at entry value ev (t bits
// | flags) as a 2x2 block per control point: dC[j] = (dCx/dPx, dCx/dPy,
// dCy/dPx, dCy/dPy).
__device__ __forceinline__ void end_point_jacobian(const CurveGeom &g, float t, uint32_t flags, bool fixed,
                                                   float4 *dC) {
    float B[4], dx, dy;
    curve_basis(g, t, B, dx, dy);
    int kind = 0;  // 0: fixed parameter, 1: on a vertical cell line, 2: on a horizontal one
    if (!fixed && !(flags & 2u)) kind = (flags & 1u) ? 2 : 1;
    if (kind == 1 && fabsf(dx) < 1e-12f) kind = 0;
    if (kind == 2 && fabsf(dy) < 1e-12f) kind = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float b = B[j];
        if (kind == 0) dC[j] = make_float4(b, 0.f, 0.f, b);
        else if (kind == 1) dC[j] = make_float4(0.f, 0.f, -(dy / dx) * b, b);
        else dC[j] = make_float4(b, -(dx / dy) * b, 0.f, 0.f);
    }
}

__device__ __forceinline__ bool filled(int w, int rule) { return rule == 0 ? (w & 0x7f) != 0 : (w & 1) != 0; }


__device__ __forceinline__ void load_curve(const CurveDesc &d, const float2 *__restrict__ tv, CurveGeom &g) {
    g.type = (int)(d.type & 0xFFu);
    g.w = g.type == kRational ? d.w : 0.f;
    const int n = g.type & 7;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float2 v = j < n ? tv[d.vpos + j] : make_float2(0.f, 0.f);
        g.px[j] = v.x;
        g.py[j] = v.y;
    }
}

// Edge-sampling adjoint of the crossings of the fragments of one merged
// group (a path's chords in one cell) with sample row r of the cell, owned
// by cell pixel column px.  J = lambda . (blend(c) - c) of the path at the
// sample of that row.
template <int S>
__device__ void crossings_adjoint(const FrameArgs &a, const DiffArgs &d, int64_t h, int px, int r, float J,
                                  int rule) {
    constexpr int WORDS = S / 8;
    const uint64_t kh = d.skey[h];
    const int w0 = (int)d.wn_scan[h];
    const float yr = ((float)r + 0.5f) / (float)(2 * S);
    for (int64_t j = h; j < d.nf && d.skey[j] == kh; ++j) {
        const uint32_t raw = d.perm[j];
        const int chg = (int32_t)d.pidw[raw] >> 30;
        if (chg == 0) continue;
        const float4 q = d.chord[raw];
        if (q.y == q.w) continue;
        uint32_t vm[4];
        vertical_mask2<S>(q.y, q.w, vm);
        if (!row_bit<S>(vm, px, r)) continue;
        const float slope = (q.z - q.x) / (q.w - q.y);
        const float lam = (yr - q.y) / (q.w - q.y);
        const float xc = q.x + (yr - q.y) * slope;
        const int pc = min(max((int)floorf(xc * 2.f), 0), 1);
        if (pc != px) continue;
        // winding just left of the crossing
        int W = w0;
        for (int64_t j2 = h; j2 < d.nf && d.skey[j2] == kh; ++j2) {
            const uint32_t raw2 = d.perm[j2];
            const int chg2 = (int32_t)d.pidw[raw2] >> 30;
            if (chg2 == 0) continue;
            uint32_t bit = 0u;
            if (j2 != j) {
                const float4 q2 = d.chord[raw2];
                if (q2.y != q2.w) {
                    uint32_t vm2[4];
                    vertical_mask2<S>(q2.y, q2.w, vm2);
                    if (row_bit<S>(vm2, px, r)) {
                        const float x2 = q2.x + (yr - q2.y) * ((q2.z - q2.x) / (q2.w - q2.y));
                        bit = xc > x2 ? 1u : 0u;
                    }
                }
            }
            uint32_t lm[4] = {0u, 0u, 0u, 0u};
#pragma unroll
            for (int w = 0; w < WORDS; ++w) lm[w] = d.lmask[(size_t)raw2 * WORDS + w];
            bit ^= row_bit<S>(lm, px, r);
            W += chg2 * (int)bit;
        }
        const bool cl = filled(W, rule), cr = filled(W + chg, rule);
        if (cl == cr) continue;
        const float dLdx = cl ? J : -J;
        // chord end points and their motion with the control points
        const int2 e0 = d.entries[raw];
        const int2 e1 = (int64_t)raw + 1 < d.nf ? d.entries[raw + 1] : make_int2(-1, 0x3f800000);
        float t0 = ffrom((uint32_t)e0.y & 0xFFFFFFFCu), t1 = ffrom((uint32_t)e1.y & 0xFFFFFFFCu);
        if (t0 < 0.f) t0 = 0.f;
        if (t1 < 0.f) t1 = 0.f;
        const bool end1 = e0.x != e1.x;
        if (end1) t1 = 1.f;
        const CurveDesc cd = a.curves[e0.x];
        CurveGeom g;
        load_curve(cd, d.tvert, g);
        float4 dC0[4], dC1[4];
        end_point_jacobian(g, t0, (uint32_t)e0.y & 3u, t0 == 0.f || t0 == 1.f, dC0);
        end_point_jacobian(g, t1, end1 ? 0u : ((uint32_t)e1.y & 3u), end1 || t1 == 0.f || t1 == 1.f, dC1);
        const int n = g.type & 7;
        for (int k = 0; k < n; ++k) {
            const float gx = (1.f - lam) * dC0[k].x + lam * dC1[k].x - slope * ((1.f - lam) * dC0[k].z + lam * dC1[k].z);
            const float gy = (1.f - lam) * dC0[k].y + lam * dC1[k].y - slope * ((1.f - lam) * dC0[k].w + lam * dC1[k].w);
            atomicAdd(&d.grad_tvert[cd.vpos + k].x, dLdx * gx);
            atomicAdd(&d.grad_tvert[cd.vpos + k].y, dLdx * gy);
        }
    }
}

struct DiffSmem {
    int4 it[kDiffChunk];
    uint4 mm[kDiffChunk];
    float4 fill[kDiffChunk];
    float acc[kDiffItemAcc][4];
};

template <int S, bool BWD>
__global__ void __launch_bounds__(kDiffThreads, 2) k_diff(FrameArgs a, DiffArgs d) {
    constexpr int SPT = S / 8;
    constexpr int WORDS = S / 8;
    __shared__ DiffSmem sm;
    __shared__ uint32_t s_bin;
    const int t = threadIdx.x;
    const int pix = t >> 3, sub = t & 7;
    const int row = pix >> 5, col = pix & 31;
    const int px_in = col & 1, k4 = px_in * 2 + row;
    const int ntx = (a.W + kTileW - 1) / kTileW;
    const size_t slot = blockIdx.x;
    for (;;) {
        __syncthreads();
        if (t == 0) s_bin = atomicAdd(d.queue, 1u);
        __syncthreads();
        const uint32_t b = s_bin;
        if ((int64_t)b >= a.n_bins) break;
        const int tile = (int)(b % ntx), crow = (int)(b / ntx);
        const int X = tile * kTileW + col, Y = crow * 2 + row;
        const bool valid = X < a.W && Y < a.H;
        const uint32_t beg = d.bstart[b], fin = d.bend[b];
        float4 c[SPT];
#pragma unroll
        for (int k = 0; k < SPT; ++k) c[k] = make_float4(1.f, 1.f, 1.f, 1.f);
        int ne = 0;
        if (BWD) {
            const int n_acc = min((int)(fin - beg), kDiffItemAcc);
            for (int i = t; i < n_acc * 4; i += kDiffThreads) (&sm.acc[0][0])[i] = 0.f;
        }
        for (uint32_t base = beg; base < fin; base += kDiffChunk) {
            __syncthreads();
            const int cnt = (int)min((uint32_t)kDiffChunk, fin - base);
            if (t < cnt) {
                const uint32_t idx = d.pval[base + t];
                const int4 it = d.draw[idx];
                sm.it[t] = it;
                if (it.w != 0) {
                    if constexpr (WORDS == 4) {
                        sm.mm[t] = reinterpret_cast<const uint4 *>(d.merged)[it.w - 1];
                    } else if constexpr (WORDS == 2) {
                        const uint2 v = reinterpret_cast<const uint2 *>(d.merged)[it.w - 1];
                        sm.mm[t] = make_uint4(v.x, v.y, 0u, 0u);
                    } else {
                        sm.mm[t] = make_uint4(d.merged[it.w - 1], 0u, 0u, 0u);
                    }
                }
                sm.fill[t] = d.fill[d.item_path[idx]];
            }
            __syncthreads();
            if (!valid) continue;
            for (int q = 0; q < cnt; ++q) {
                const int4 it = sm.it[q];
                const int x = (int)((uint32_t)it.x & 0xFFFFu);
                const bool frag = it.w != 0;
                const int len = frag ? 2 : it.y;
                if (X < x || X >= x + len) continue;
                const uint32_t m = frag ? pixel_mask(sm.mm[q], S, k4) : 0xFFFFFFFFu;
                const float4 f = sm.fill[q];
                const float om = 1.f - f.w;
                uint32_t cov = 0u;
#pragma unroll
                for (int k = 0; k < SPT; ++k) cov |= ((m >> (sub + 8 * k)) & 1u) << k;
                if (BWD) {
                    if (ne < d.tape_depth) {
                        const size_t e = slot * (size_t)d.tape_depth + ne;
                        d.tape_item[e * kDiffThreads + t] = (base - beg + (uint32_t)q) | (cov << 24);
#pragma unroll
                        for (int k = 0; k < SPT; ++k) d.tape[(e * SPT + k) * kDiffThreads + t] = c[k];
                    } else {
                        atomicOr(d.status, 1u);
                    }
                    ++ne;
                }
#pragma unroll
                for (int k = 0; k < SPT; ++k) {
                    if ((cov >> k) & 1u) {
                        c[k].x = f.x * f.w + c[k].x * om;
                        c[k].y = f.y * f.w + c[k].y * om;
                        c[k].z = f.z * f.w + c[k].z * om;
                        c[k].w = f.w * f.w + c[k].w * om;
                    }
                }
            }
        }
        if (!BWD) {
            float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int k = 0; k < SPT; ++k) {
                sum.x += c[k].x;
                sum.y += c[k].y;
                sum.z += c[k].z;
                sum.w += c[k].w;
            }
#pragma unroll
            for (int o = 1; o < 8; o <<= 1) {
                sum.x += __shfl_xor_sync(0xffffffffu, sum.x, o);
                sum.y += __shfl_xor_sync(0xffffffffu, sum.y, o);
                sum.z += __shfl_xor_sync(0xffffffffu, sum.z, o);
                sum.w += __shfl_xor_sync(0xffffffffu, sum.w, o);
            }
            if (valid && sub == 0) {
                const float inv = 1.f / (float)S;
                d.image[(int64_t)Y * a.W + X] = make_float4(sum.x * inv, sum.y * inv, sum.z * inv, sum.w * inv);
            }
            continue;
        }
        // ---- reverse sweep
        if (valid && ne <= d.tape_depth) {
            const float inv = 1.f / (float)S;
            const float4 G = d.grad_image[(int64_t)Y * a.W + X];
            float4 lam[SPT];
#pragma unroll
            for (int k = 0; k < SPT; ++k) lam[k] = make_float4(G.x * inv, G.y * inv, G.z * inv, G.w * inv);
            for (int e0 = ne - 1; e0 >= 0; --e0) {
                const size_t e = slot * (size_t)d.tape_depth + e0;
                const uint32_t rec = d.tape_item[e * kDiffThreads + t];
                const uint32_t q = rec & 0xFFFFFFu, cov = rec >> 24;
                const uint32_t idx = d.pval[beg + q];
                const int4 it = d.draw[idx];
                const uint32_t path = d.item_path[idx];
                const float4 f = d.fill[path];
                const float av = f.w, om = 1.f - av;
                float4 gf = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int k = 0; k < SPT; ++k) {
                    const float4 cb = d.tape[(e * SPT + k) * kDiffThreads + t];
                    const float4 l = lam[k];
                    const float J = l.x * av * (f.x - cb.x) + l.y * av * (f.y - cb.y) + l.z * av * (f.z - cb.z) +
                                    l.w * av * (av - cb.w);
                    if ((cov >> k) & 1u) {
                        gf.x += l.x * av;
                        gf.y += l.y * av;
                        gf.z += l.z * av;
                        gf.w += l.x * (f.x - cb.x) + l.y * (f.y - cb.y) + l.z * (f.z - cb.z) + l.w * (2.f * av - cb.w);
                        lam[k] = make_float4(l.x * om, l.y * om, l.z * om, l.w * om);
                    }
                    if (it.w != 0 && J != 0.f)
                        crossings_adjoint<S>(a, d, d.heads[it.w - 1], px_in, row * S + sub + 8 * k, J,
                                             a.fill_rule[path]);
                }
                if (gf.x != 0.f || gf.y != 0.f || gf.z != 0.f || gf.w != 0.f) {
                    if (q < (uint32_t)kDiffItemAcc) {
                        atomicAdd(&sm.acc[q][0], gf.x);
                        atomicAdd(&sm.acc[q][1], gf.y);
                        atomicAdd(&sm.acc[q][2], gf.z);
                        atomicAdd(&sm.acc[q][3], gf.w);
                    } else {
                        atomicAdd(&d.grad_fill[path].x, gf.x);
                        atomicAdd(&d.grad_fill[path].y, gf.y);
                        atomicAdd(&d.grad_fill[path].z, gf.z);
                        atomicAdd(&d.grad_fill[path].w, gf.w);
                    }
                }
            }
        }
        __syncthreads();
        const int n_acc = min((int)(fin - beg), kDiffItemAcc);
        for (int q = t; q < n_acc; q += kDiffThreads) {
            const float *v = sm.acc[q];
            if (v[0] == 0.f && v[1] == 0.f && v[2] == 0.f && v[3] == 0.f) continue;
            const uint32_t path = d.item_path[d.pval[beg + q]];
            atomicAdd(&d.grad_fill[path].x, v[0]);
            atomicAdd(&d.grad_fill[path].y, v[1]);
            atomicAdd(&d.grad_fill[path].z, v[2]);
            atomicAdd(&d.grad_fill[path].w, v[3]);
        }
    }
}

// dL/d(transformed vertex) -> dL/d(input vertex) and dL/d(path affine),
// through k_transform's map (affine, 4x4 with the projective divide, the
// depth fold; the integer-x nudge has unit derivative).
__global__ void k_diff_vertex(FrameArgs a, const float2 *__restrict__ gt, const uint32_t *__restrict__ vmap,
                              float2 *__restrict__ gv, float *__restrict__ ga) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.V) return;
    const float2 g = gt[i];
    const float2 p = a.vertex[i];
    const uint32_t pid = a.vertex_pid[i];
    float xa = p.x, ya = p.y;
    float A[6] = {1.f, 0.f, 0.f, 1.f, 0.f, 0.f};
    if (a.affine) {
#pragma unroll
        for (int k = 0; k < 6; ++k) A[k] = a.affine[6 * (size_t)pid + k];
        xa = A[0] * p.x + A[2] * p.y + A[4];
        ya = A[1] * p.x + A[3] * p.y + A[5];
    }
    float ov[4], dox[4], doy[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        ov[r] = a.m[4 * r] * xa + a.m[4 * r + 1] * ya + a.m[4 * r + 3];
        dox[r] = a.m[4 * r];
        doy[r] = a.m[4 * r + 1];
    }
    float q[3], qx[3], qy[3];
    const float i3 = 1.f / ov[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        q[r] = ov[r] * i3;
        qx[r] = (dox[r] - q[r] * dox[3]) * i3;
        qy[r] = (doy[r] - q[r] * doy[3]) * i3;
    }
    const float w = (float)a.W, h = (float)a.H, z = (float)min(a.W, a.H);
    const float cutoff = -z * 0.5f;
    if (q[2] < cutoff) {
        q[2] = cutoff;
        qx[2] = qy[2] = 0.f;
    }
    const float den = q[2] + z, f = z / den;
    // d(out)/d(xa, ya): out.x = (q0 - w/2) f + w/2, out.y = (q1 - h/2) f + h/2
    const float fx = -f / den * qx[2], fy = -f / den * qy[2];
    const float Jxx = qx[0] * f + (q[0] - w * .5f) * fx, Jxy = qy[0] * f + (q[0] - w * .5f) * fy;
    const float Jyx = qx[1] * f + (q[1] - h * .5f) * fx, Jyy = qy[1] * f + (q[1] - h * .5f) * fy;
    const float gxa = Jxx * g.x + Jyx * g.y, gya = Jxy * g.x + Jyy * g.y;
    gv[vmap[i]] = make_float2(A[0] * gxa + A[1] * gya, A[2] * gxa + A[3] * gya);
    if (a.affine && ga && (gxa != 0.f || gya != 0.f)) {
        float *G = ga + 6 * (size_t)pid;
        atomicAdd(G + 0, gxa * p.x);
        atomicAdd(G + 1, gya * p.x);
        atomicAdd(G + 2, gxa * p.y);
        atomicAdd(G + 3, gya * p.y);
        atomicAdd(G + 4, gxa);
        atomicAdd(G + 5, gya);
    }
}

int diff_sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
    }
    return n;
}

template <bool BWD>
int launch_diff(const FrameArgs &a, const DiffArgs &d, cudaStream_t s) {
    if (a.n_bins <= 0) return 0;
    cudaMemsetAsync(d.queue, 0, sizeof(uint32_t), s);
    const unsigned grid = (unsigned)diff_blocks(a);
    if (a.S == 8) k_diff<8, BWD><<<grid, kDiffThreads, 0, s>>>(a, d);
    else if (a.S == 16) k_diff<16, BWD><<<grid, kDiffThreads, 0, s>>>(a, d);
    else k_diff<32, BWD><<<grid, kDiffThreads, 0, s>>>(a, d);
    return 1;
}

}  // namespace

int64_t diff_blocks(const FrameArgs &a) {
    return std::max<int64_t>(1, std::min<int64_t>(a.n_bins, (int64_t)diff_sm_count() * 2));
}

int64_t diff_tape_words(const FrameArgs &a, int depth) {
    return diff_blocks(a) * (int64_t)depth * (a.S / 8) * kDiffThreads;
}

int launch_diff_forward(const FrameArgs &a, const DiffArgs &d, cudaStream_t s) { return launch_diff<false>(a, d, s); }

int launch_diff_backward(const FrameArgs &a, const DiffArgs &d, cudaStream_t s) { return launch_diff<true>(a, d, s); }

int launch_diff_vertex(const FrameArgs &a, const float2 *grad_tvert, const uint32_t *vmap, float2 *grad_vertex,
                       float *grad_affine, cudaStream_t s) {
    if (a.V <= 0) return 0;
    k_diff_vertex<<<(unsigned)((a.V + 255) / 256), 256, 0, s>>>(a, grad_tvert, vmap, grad_vertex, grad_affine);
    return 1;
}

}  // namespace spr
