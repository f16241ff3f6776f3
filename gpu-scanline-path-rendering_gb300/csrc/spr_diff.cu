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

constexpr int kDiffThreads = 256;    // 8 warps, each working on its own cells
constexpr int kDiffPathAcc = 4096;   // paths with shared-memory fill-gradient accumulators (backward)
constexpr int kDiffCacheSlots = 256; // else: slots of each warp's path-gradient cache
constexpr int kTileW = kBinW;  // columns of a resolve bin

__device__ __forceinline__ uint32_t pixel_mask(const uint4 &mm, int S, int k) {
    if (S == 32) return k == 0 ? mm.x : (k == 1 ? mm.y : (k == 2 ? mm.z : mm.w));
    if (S == 16) return ((k < 2 ? mm.x : mm.y) >> (16 * (k & 1))) & 0xFFFFu;
    return (mm.x >> (8 * k)) & 0xFFu;
}

// Bit r of the 2S stacked sample rows of cell column px in a vertical-mask
// word layout (vertical_mask / vertical_mask2).  The word is picked by
// selects: px and r vary by lane, and a lane-dependent array index would
// put the fragment's masks in local memory.
template <int S>
__device__ __forceinline__ uint32_t row_bit(const uint32_t *m, int px, int r) {
    if constexpr (S == 32) {
        const int i = 2 * px + (r >> 5);
        const uint32_t w = i < 2 ? (i == 0 ? m[0] : m[1]) : (i == 2 ? m[2] : m[3]);
        return (w >> (r & 31)) & 1u;
    } else if constexpr (S == 16) {
        return ((px ? m[1] : m[0]) >> r) & 1u;
    } else {
        return (m[0] >> r) & 1u;
    }
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

// Warp sums of N values (N = 2, 4, 8), returned to every lane: a
// reduce-scatter in which a lane keeps, at the exchange across lane bit O, the
// half of its partial sums that its side owns (M values), then plain
// butterflies over the remaining lane bits and one broadcast per value; value
// i ends in lane i * 32 / N.  2N + 4 - log2(N) shuffles instead of 5N.
template <int M, int O, int N>
__device__ __forceinline__ void reduce_scatter(float (&t)[N], int lane) {
    if constexpr (M >= 1) {
        const bool hi = (lane & O) != 0;
#pragma unroll
        for (int i = 0; i < M; ++i) {
            const float keep = hi ? t[M + i] : t[i];
            const float send = hi ? t[i] : t[M + i];
            t[i] = keep + __shfl_xor_sync(0xffffffffu, send, O);
        }
        reduce_scatter<M / 2, O / 2, N>(t, lane);
    } else {
#pragma unroll
        for (int o = O; o >= 1; o >>= 1) t[0] += __shfl_xor_sync(0xffffffffu, t[0], o);
    }
}

template <int N>
__device__ __forceinline__ void warp_sums(float (&v)[N], int lane) {
    float t[N];
#pragma unroll
    for (int i = 0; i < N; ++i) t[i] = v[i];
    reduce_scatter<N / 2, 16, N>(t, lane);
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = __shfl_sync(0xffffffffu, t[0], i * (32 / N));
}

__device__ __forceinline__ float4 warp_sum4(float4 x, int lane) {
    float v[4] = {x.x, x.y, x.z, x.w};
    warp_sums<4>(v, lane);
    return make_float4(v[0], v[1], v[2], v[3]);
}

// One fragment of a merged group, held by one lane of the cell's warp.
template <int S>
struct GroupFrag {
    float4 q;          // chord in cell units: x0, y0, slope dx/dy (0 when horizontal), y1
    uint32_t vm[S / 8];  // rows between the chord's end points
    uint32_t lm[S / 8];  // left mask
    int chg;           // winding change (0: no contribution)
    uint32_t raw;
};

template <int S>
__device__ __forceinline__ void load_group_frag(const DiffArgs &d, int64_t j, GroupFrag<S> &f) {
    constexpr int WORDS = S / 8;
    f.raw = d.perm[j];
    f.chg = (int32_t)d.pidw[f.raw] >> 30;
    const float4 c = d.chord[f.raw];
    f.q = make_float4(c.x, c.y, c.w != c.y ? (c.z - c.x) / (c.w - c.y) : 0.f, c.w);
#pragma unroll
    for (int w = 0; w < WORDS; ++w) {
        f.vm[w] = d.vmask[(size_t)f.raw * WORDS + w];
        f.lm[w] = d.lmask[(size_t)f.raw * WORDS + w];
    }
}

template <int S>
__device__ __forceinline__ GroupFrag<S> shfl_frag(const GroupFrag<S> &f, int src) {
    GroupFrag<S> o;
    o.q.x = __shfl_sync(0xffffffffu, f.q.x, src);
    o.q.y = __shfl_sync(0xffffffffu, f.q.y, src);
    o.q.z = __shfl_sync(0xffffffffu, f.q.z, src);
    o.q.w = __shfl_sync(0xffffffffu, f.q.w, src);
#pragma unroll
    for (int w = 0; w < S / 8; ++w) {
        o.vm[w] = __shfl_sync(0xffffffffu, f.vm[w], src);
        o.lm[w] = __shfl_sync(0xffffffffu, f.lm[w], src);
    }
    o.chg = __shfl_sync(0xffffffffu, f.chg, src);
    o.raw = __shfl_sync(0xffffffffu, f.raw, src);
    return o;
}

// Chain of one fragment's crossings to its curve's control points: the
// crossings contribute sum dL/dx * ((1 - lam) dC0 + lam dC1) projected on x
// at fixed y, i.e. A * (dC0x - s dC0y) + B * (dC1x - s dC1y).
__device__ void fragment_chain(const FrameArgs &a, const DiffArgs &d, uint32_t raw, float slope, float A, float B) {
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
        const float gx = A * (dC0[k].x - slope * dC0[k].z) + B * (dC1[k].x - slope * dC1[k].z);
        const float gy = A * (dC0[k].y - slope * dC0[k].w) + B * (dC1[k].y - slope * dC1[k].w);
        atomicAdd(&d.grad_tvert[cd.vpos + k].x, gx);
        atomicAdd(&d.grad_tvert[cd.vpos + k].y, gy);
    }
}

// Edge-sampling adjoint of one merged group (a path's chords in one cell)
// for the cell's warp.  Lane l holds samples sub + 8k of cell pixel k4 =
// l >> 3 and J[k] = lambda . (blend(c) - c) of the path at those samples.
// Groups are loaded 32 fragments at a time, one per lane, and broadcast by
// shuffles; every shuffle is executed by the whole warp.
template <int S>
__device__ void group_adjoint(const FrameArgs &a, const DiffArgs &d, int64_t h, int rule, const float *J, int lane) {
    constexpr int SPT = S / 8;
    const int k4 = lane >> 3, sub = lane & 7, px = k4 >> 1, py = k4 & 1;
    const int w0 = (int)d.wn_scan[h];
    // group size: the run of equal keys from h, 32 keys per step
    const uint64_t kh = d.skey[h] & kKeyMask;
    int gs = 0;
    for (;;) {
        const int64_t j = h + gs + lane;
        const uint32_t ends = __ballot_sync(0xffffffffu, j >= d.nf || (d.skey[j] & kKeyMask) != kh);
        if (ends) {
            gs += __ffs(ends) - 1;
            break;
        }
        gs += 32;
    }
    for (int base = 0; base < gs; base += 32) {
        const int nw = min(32, gs - base);
        GroupFrag<S> mine;
        if (lane < nw) load_group_frag<S>(d, h + base + lane, mine);
        else mine = GroupFrag<S>{};
        for (int j = 0; j < nw; ++j) {
            const GroupFrag<S> f = shfl_frag<S>(mine, j);
            if (f.chg == 0 || f.q.y == f.q.w) continue;  // uniform
            const float slope = f.q.z;
            bool cand[SPT];
            float xc[SPT], yr[SPT];
            int W[SPT];
            bool any = false;
#pragma unroll
            for (int k = 0; k < SPT; ++k) {
                const int r = py * S + sub + 8 * k;
                yr[k] = ((float)r + 0.5f) / (float)(2 * S);
                xc[k] = f.q.x + (yr[k] - f.q.y) * slope;
                const int pc = min(max((int)floorf(xc[k] * 2.f), 0), 1);
                cand[k] = J[k] != 0.f && row_bit<S>(f.vm, px, r) && pc == px;
                W[k] = w0;
                any |= cand[k];
            }
            if (!__any_sync(0xffffffffu, any)) continue;
            // winding just left of each candidate crossing: this window by shuffles ...
            for (int j2 = 0; j2 < nw; ++j2) {
                const GroupFrag<S> f2 = shfl_frag<S>(mine, j2);
                if (f2.chg == 0) continue;  // uniform
#pragma unroll
                for (int k = 0; k < SPT; ++k) {
                    const int r = py * S + sub + 8 * k;
                    uint32_t bit = 0u;
                    if (j2 != j && row_bit<S>(f2.vm, px, r)) {
                        const float x2 = f2.q.x + (yr[k] - f2.q.y) * f2.q.z;
                        bit = xc[k] > x2 ? 1u : 0u;
                    }
                    bit ^= row_bit<S>(f2.lm, px, r);
                    W[k] += f2.chg * (int)bit;
                }
            }
            // ... and the other windows of a group of more than 32 fragments from memory
            if (gs > 32 && any) {
                for (int j2 = 0; j2 < gs; ++j2) {
                    if (j2 >= base && j2 < base + nw) continue;
                    GroupFrag<S> f2;
                    load_group_frag<S>(d, h + j2, f2);
                    if (f2.chg == 0) continue;
#pragma unroll
                    for (int k = 0; k < SPT; ++k) {
                        const int r = py * S + sub + 8 * k;
                        uint32_t bit = 0u;
                        if (row_bit<S>(f2.vm, px, r)) {
                            const float x2 = f2.q.x + (yr[k] - f2.q.y) * f2.q.z;
                            bit = xc[k] > x2 ? 1u : 0u;
                        }
                        bit ^= row_bit<S>(f2.lm, px, r);
                        W[k] += f2.chg * (int)bit;
                    }
                }
            }
            float sA = 0.f, sB = 0.f;
#pragma unroll
            for (int k = 0; k < SPT; ++k) {
                if (!cand[k]) continue;
                const bool cl = filled(W[k], rule), cr = filled(W[k] + f.chg, rule);
                if (cl == cr) continue;
                const float g = cl ? J[k] : -J[k];
                const float lam = (yr[k] - f.q.y) / (f.q.w - f.q.y);
                sA += g * (1.f - lam);
                sB += g * lam;
            }
            float sAB[2] = {sA, sB};
            warp_sums<2>(sAB, lane);
            sA = sAB[0];
            sB = sAB[1];
            if (lane == 0 && (sA != 0.f || sB != 0.f)) {
                const uint32_t n = atomicAdd(d.n_chain, 1u);
                if ((int64_t)n < d.nf) d.chain[n] = make_float4(__uint_as_float(f.raw), slope, sA, sB);
                else atomicOr(d.status, 2u);
            }
        }
    }
}

__device__ __forceinline__ uint4 load_merged(const uint32_t *merged, int words, uint32_t g) {
    if (words == 4) return reinterpret_cast<const uint4 *>(merged)[g];
    if (words == 2) {
        const uint2 v = reinterpret_cast<const uint2 *>(merged)[g];
        return make_uint4(v.x, v.y, 0u, 0u);
    }
    return make_uint4(merged[g], 0u, 0u, 0u);
}

__device__ __forceinline__ void global_fill_grad(const DiffArgs &d, uint32_t path, float4 g) {
    atomicAdd(&d.grad_fill[path].x, g.x);
    atomicAdd(&d.grad_fill[path].y, g.y);
    atomicAdd(&d.grad_fill[path].z, g.z);
    atomicAdd(&d.grad_fill[path].w, g.w);
}

// A fill gradient (lane 0 of the warp): into the block's per-path
// accumulators (acc) when every path has one; else into the warp's
// direct-mapped cache (slot = path mod kDiffCacheSlots, tag = path), whose
// evicted entries go to the global gradient.  Neighbouring cells share most
// of their paths, so the cache turns most global atomics into register adds.
__device__ __forceinline__ void add_fill_grad(const DiffArgs &d, float4 *acc, float4 *cache, uint32_t *tag,
                                              uint32_t path, float4 g) {
    if (cache != nullptr) {
        const uint32_t slot = path & (kDiffCacheSlots - 1);
        const uint32_t t = tag[slot];
        if (t == path) {
            float4 &v = cache[slot];
            v.x += g.x;
            v.y += g.y;
            v.z += g.z;
            v.w += g.w;
        } else {
            if (t != 0xFFFFFFFFu) global_fill_grad(d, t, cache[slot]);
            cache[slot] = g;
            tag[slot] = path;
        }
    } else if (acc != nullptr) {
        atomicAdd(&acc[path].x, g.x);
        atomicAdd(&acc[path].y, g.y);
        atomicAdd(&acc[path].z, g.z);
        atomicAdd(&acc[path].w, g.w);
    } else {
        global_fill_grad(d, path, g);
    }
}

// The scene of resolve bin b: viewport, the bin index within the scene and
// the scene's first pixel (batch frames; a single scene otherwise).
struct BinScene {
    int W, H;
    uint32_t lb;
    int64_t image_off;
};
__device__ __forceinline__ BinScene bin_scene(const FrameArgs &a, uint32_t b) {
    BinScene r{a.W, a.H, b, 0};
    if (a.scenes != nullptr) {
        int lo = 0, hi = a.n_scenes - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (a.scenes[mid].bin_off <= b) lo = mid;
            else hi = mid - 1;
        }
        const SceneInfo *sc = a.scenes + lo;
        r.W = sc->W;
        r.H = sc->H;
        r.lb = b - sc->bin_off;
        r.image_off = sc->image_off;
    }
    return r;
}

// The items of the resolve pairs in bin order, one contiguous record each.
__global__ void k_diff_gather(DiffArgs d, int words) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.npairs) return;
    const uint32_t idx = d.pval[p];
    const int4 it = d.draw[idx];
    const uint32_t path = d.item_path[idx];
    d.bitem[p] = make_uint4((uint32_t)it.x, (uint32_t)it.y, (uint32_t)it.w, path);
    d.bfill[p] = d.fill[path];
    d.bmm[p] = it.w != 0 ? load_merged(d.merged, words, (uint32_t)it.w - 1u) : make_uint4(0u, 0u, 0u, 0u);
}

// The crossing sums of every fragment chained to its curve's control points.
__global__ void k_diff_chain(FrameArgs a, DiffArgs d) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)min((uint64_t)*d.n_chain, (uint64_t)d.nf)) return;
    const float4 r = d.chain[i];
    fragment_chain(a, d, __float_as_uint(r.x), r.y, r.z, r.w);
}

// Persistent warps over (bin, cell) units from a queue: warp = one cell of a
// bin, lane l = pixel k4 = l >> 3 of the cell (k4 = px * 2 + py), samples
// (l & 7) + 8k.  Every item touching a cell touches all its pixels, so the
// walk over the bin's items is warp-uniform; the items are read 32 at a time
// (one per lane), the touching ones found by a ballot and broadcast.  Warps
// never wait for one another.
template <int S, bool BWD, bool CACHE>
__global__ void __launch_bounds__(kDiffThreads, 3) k_diff(FrameArgs a, DiffArgs d) {
    constexpr int SPT = S / 8;
    constexpr int WORDS = S / 8;
    extern __shared__ float4 s_acc[];  // fill-gradient accumulators (backward)
    const int lane = threadIdx.x & 31;
    const int k4 = lane >> 3, sub = lane & 7;
    const int px_in = k4 >> 1, py_in = k4 & 1;
    const size_t wslot = (size_t)blockIdx.x * (kDiffThreads / 32) + (threadIdx.x >> 5);
    // fill-gradient accumulators: per path for the block (few paths), else
    // (CACHE) a path cache per warp: values, then tags
    float4 *acc = (BWD && !CACHE) ? s_acc : nullptr;
    float4 *cache = (BWD && CACHE) ? s_acc + (threadIdx.x >> 5) * kDiffCacheSlots : nullptr;
    uint32_t *tag = (BWD && CACHE) ? reinterpret_cast<uint32_t *>(s_acc + (kDiffThreads / 32) * kDiffCacheSlots) +
                                         (threadIdx.x >> 5) * kDiffCacheSlots
                                   : nullptr;
    if (acc)
        for (int i = threadIdx.x; i < a.P; i += kDiffThreads) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (tag)
        for (int i = lane; i < kDiffCacheSlots; i += 32) tag[i] = 0xFFFFFFFFu;
    if (BWD) __syncthreads();
    const int64_t n_units = a.n_bins * (kTileW / 2);
    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(d.queue, 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if ((int64_t)u >= n_units) break;
        const uint32_t b = u / (kTileW / 2);
        const int cw = (int)(u % (kTileW / 2));
        const BinScene bs = bin_scene(a, b);
        const int ntx = (bs.W + kTileW - 1) / kTileW;
        const int tile = (int)(bs.lb % ntx), crow = (int)(bs.lb / ntx);
        const int cellx = tile * kTileW + 2 * cw;
        if (cellx >= bs.W) continue;
        const int X = cellx + px_in, Y = crow * 2 + py_in;
        const bool valid = X < bs.W && Y < bs.H;
        const int64_t pix = bs.image_off + (int64_t)Y * bs.W + X;
        const uint32_t beg = d.bstart[b], fin = d.bend[b];
        float4 c[SPT];
#pragma unroll
        for (int k = 0; k < SPT; ++k) c[k] = make_float4(1.f, 1.f, 1.f, 1.f);
        // backward tape: ne item records; nsl sample-state slots (the state
        // before every fragment and at the start of every run of spans)
        int ne = 0, nsl = 0, run_slot = -1;
        float ralpha = 1.f;
        float4 rbeta = make_float4(0.f, 0.f, 0.f, 0.f);
        const size_t rbase = wslot * (size_t)d.tape_depth;
        // the bin's items, 32 at a time (lane l holds item base + l), the next
        // chunk loaded while the current one is applied
        uint4 it = make_uint4(0u, 0u, 0u, 0u), my_mm = it;
        float4 my_fill = make_float4(0.f, 0.f, 0.f, 0.f);
        if (beg + lane < fin) {
            it = d.bitem[beg + lane];
            my_fill = d.bfill[beg + lane];
            my_mm = d.bmm[beg + lane];
        }
        for (uint32_t base = beg; base < fin; base += 32) {
            uint4 nit = make_uint4(0u, 0u, 0u, 0u), nmm = nit;
            float4 nfill = make_float4(0.f, 0.f, 0.f, 0.f);
            if (base + 32 + lane < fin) {
                nit = d.bitem[base + 32 + lane];
                nfill = d.bfill[base + 32 + lane];
                nmm = d.bmm[base + 32 + lane];
            }
            bool touch = false;
            if (base + lane < fin) {
                const int x = (int)(it.x & 0xFFFFu);
                touch = it.z != 0u ? x == cellx : (cellx >= x && cellx < x + (int)it.y);
            }
            uint32_t tm = __ballot_sync(0xffffffffu, touch);
            while (tm) {
                const int q = __ffs(tm) - 1;
                tm &= tm - 1u;
                const uint32_t w = __shfl_sync(0xffffffffu, it.z, q);
                const uint32_t path = __shfl_sync(0xffffffffu, it.w, q);
                float4 f;
                f.x = __shfl_sync(0xffffffffu, my_fill.x, q);
                f.y = __shfl_sync(0xffffffffu, my_fill.y, q);
                f.z = __shfl_sync(0xffffffffu, my_fill.z, q);
                f.w = __shfl_sync(0xffffffffu, my_fill.w, q);
                const bool frag = w != 0;
                uint32_t m = 0xFFFFFFFFu;
                if (frag) {
                    uint4 mm;
                    mm.x = __shfl_sync(0xffffffffu, my_mm.x, q);
                    mm.y = WORDS > 1 ? __shfl_sync(0xffffffffu, my_mm.y, q) : 0u;
                    mm.z = WORDS > 2 ? __shfl_sync(0xffffffffu, my_mm.z, q) : 0u;
                    mm.w = WORDS > 2 ? __shfl_sync(0xffffffffu, my_mm.w, q) : 0u;
                    m = pixel_mask(mm, S, k4);
                }
                const float om = 1.f - f.w;
                // A run of spans (which cover every sample of the cell) is
                // carried as c = ralpha * c_run + rbeta, c_run the samples'
                // state where the run starts; states are materialized at
                // fragments and at the end.
                if (frag && run_slot >= 0) {
#pragma unroll
                    for (int k = 0; k < SPT; ++k)
                        c[k] = make_float4(ralpha * c[k].x + rbeta.x, ralpha * c[k].y + rbeta.y,
                                           ralpha * c[k].z + rbeta.z, ralpha * c[k].w + rbeta.w);
                    run_slot = -1;
                }
                int sidx = run_slot;
                if (frag || run_slot < 0) {
                    sidx = nsl++;
                    if (BWD && sidx < d.tape_depth) {
                        const size_t e = rbase + sidx;
#pragma unroll
                        for (int k = 0; k < SPT; ++k) d.tape[(e * SPT + k) * 32 + lane] = c[k];
                    }
                    if (!frag) {
                        run_slot = sidx;
                        ralpha = 1.f;
                        rbeta = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                }
                if (BWD) {
                    if (ne < d.tape_depth) {
                        if (lane == 0) {
                            float4 *rec = d.tape_rec + (rbase + ne) * 3;
                            rec[0] = f;
                            rec[1] = rbeta;
                            rec[2] = make_float4(ralpha, __uint_as_float(path), __uint_as_float(w),
                                                 __uint_as_float((uint32_t)sidx));
                        }
                    } else if (lane == 0) {
                        atomicOr(d.status, 1u);
                    }
                    ++ne;
                }
                if (!frag) {  // the run's composition up to and including this span
                    rbeta = make_float4(f.x * f.w + rbeta.x * om, f.y * f.w + rbeta.y * om, f.z * f.w + rbeta.z * om,
                                        f.w * f.w + rbeta.w * om);
                    ralpha *= om;
                } else {
#pragma unroll
                    for (int k = 0; k < SPT; ++k) {
                        if ((m >> (sub + 8 * k)) & 1u) {
                            c[k].x = f.x * f.w + c[k].x * om;
                            c[k].y = f.y * f.w + c[k].y * om;
                            c[k].z = f.z * f.w + c[k].z * om;
                            c[k].w = f.w * f.w + c[k].w * om;
                        }
                    }
                }
            }
            it = nit;
            my_fill = nfill;
            my_mm = nmm;
        }
        if (run_slot >= 0) {
#pragma unroll
            for (int k = 0; k < SPT; ++k)
                c[k] = make_float4(ralpha * c[k].x + rbeta.x, ralpha * c[k].y + rbeta.y, ralpha * c[k].z + rbeta.z,
                                   ralpha * c[k].w + rbeta.w);
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
                const float inv = d.out_scale / (float)S;
                float4 v = make_float4(sum.x * inv, sum.y * inv, sum.z * inv, sum.w * inv);
                if (d.accumulate) {
                    const float4 o = d.image[pix];
                    v = make_float4(o.x + v.x, o.y + v.y, o.z + v.z, o.w + v.w);
                }
                d.image[pix] = v;
            }
            continue;
        }
        // ---- reverse sweep (warp-uniform)
        if (ne > d.tape_depth || nsl > d.tape_depth) continue;
        const float inv = d.out_scale / (float)S;
        const float4 G = valid ? d.grad_image[pix] : make_float4(0.f, 0.f, 0.f, 0.f);
        float4 lam[SPT];
#pragma unroll
        for (int k = 0; k < SPT; ++k) lam[k] = make_float4(G.x * inv, G.y * inv, G.z * inv, G.w * inv);
        int cur_slot = -1;  // run being swept (its start slot), -1 outside runs
        float pi = 1.f;
        float4 Lsum = make_float4(0.f, 0.f, 0.f, 0.f), Ksum = Lsum;
        float4 rf = make_float4(0.f, 0.f, 0.f, 0.f), rbb = rf, rr2 = rf;  // lane l: record e_hi - l
        for (int e0 = ne - 1; e0 >= 0; --e0) {
            const int jl = (ne - 1 - e0) & 31;
            if (jl == 0) {  // the next 32 records, one per lane
                if (e0 - lane >= 0) {
                    const float4 *rec = d.tape_rec + (rbase + e0 - lane) * 3;
                    rf = rec[0];
                    rbb = rec[1];
                    rr2 = rec[2];
                }
            }
            float4 f, rb, r2;
            f.x = __shfl_sync(0xffffffffu, rf.x, jl);
            f.y = __shfl_sync(0xffffffffu, rf.y, jl);
            f.z = __shfl_sync(0xffffffffu, rf.z, jl);
            f.w = __shfl_sync(0xffffffffu, rf.w, jl);
            rb.x = __shfl_sync(0xffffffffu, rbb.x, jl);
            rb.y = __shfl_sync(0xffffffffu, rbb.y, jl);
            rb.z = __shfl_sync(0xffffffffu, rbb.z, jl);
            rb.w = __shfl_sync(0xffffffffu, rbb.w, jl);
            r2.x = __shfl_sync(0xffffffffu, rr2.x, jl);
            r2.y = __shfl_sync(0xffffffffu, rr2.y, jl);
            r2.z = __shfl_sync(0xffffffffu, rr2.z, jl);
            r2.w = __shfl_sync(0xffffffffu, rr2.w, jl);
            const float ra = r2.x;
            const uint32_t path = __float_as_uint(r2.y), w = __float_as_uint(r2.z);
            const int sidx = (int)__float_as_uint(r2.w);
            const float av = f.w, om = 1.f - av;
            if (w == 0u) {
                // span: every sample covered; inside a run the samples' adjoints
                // are the run end's times the scalar pi, so the fill gradient
                // needs only the run's sums Lsum = sum lambda and Ksum = sum
                // lambda * c_run (c before the span = ra * c_run + rb).
                if (sidx != cur_slot) {
                    if (cur_slot >= 0) {
#pragma unroll
                        for (int k = 0; k < SPT; ++k)
                            lam[k] = make_float4(lam[k].x * pi, lam[k].y * pi, lam[k].z * pi, lam[k].w * pi);
                    }
                    const size_t es = rbase + sidx;
                    float4 ls = make_float4(0.f, 0.f, 0.f, 0.f), ks = ls;
#pragma unroll
                    for (int k = 0; k < SPT; ++k) {
                        const float4 cr = d.tape[(es * SPT + k) * 32 + lane];
                        ls.x += lam[k].x;
                        ls.y += lam[k].y;
                        ls.z += lam[k].z;
                        ls.w += lam[k].w;
                        ks.x += lam[k].x * cr.x;
                        ks.y += lam[k].y * cr.y;
                        ks.z += lam[k].z * cr.z;
                        ks.w += lam[k].w * cr.w;
                    }
                    float lk[8] = {ls.x, ls.y, ls.z, ls.w, ks.x, ks.y, ks.z, ks.w};
                    warp_sums<8>(lk, lane);
                    Lsum = make_float4(lk[0], lk[1], lk[2], lk[3]);
                    Ksum = make_float4(lk[4], lk[5], lk[6], lk[7]);
                    cur_slot = sidx;
                    pi = 1.f;
                }
                const float cx = ra * Ksum.x + rb.x * Lsum.x, cy = ra * Ksum.y + rb.y * Lsum.y;
                const float cz = ra * Ksum.z + rb.z * Lsum.z, cw = ra * Ksum.w + rb.w * Lsum.w;
                const float4 gf = make_float4(
                    pi * av * Lsum.x, pi * av * Lsum.y, pi * av * Lsum.z,
                    pi * (Lsum.x * f.x - cx + Lsum.y * f.y - cy + Lsum.z * f.z - cz + 2.f * av * Lsum.w - cw));
                if (lane == 0 && (gf.x != 0.f || gf.y != 0.f || gf.z != 0.f || gf.w != 0.f))
                    add_fill_grad(d, acc, cache, tag, path, gf);
                pi *= om;
                continue;
            }
            // fragment: per-sample coverage; first close a pending run
            if (cur_slot >= 0) {
#pragma unroll
                for (int k = 0; k < SPT; ++k)
                    lam[k] = make_float4(lam[k].x * pi, lam[k].y * pi, lam[k].z * pi, lam[k].w * pi);
                cur_slot = -1;
            }
            const uint32_t m = pixel_mask(load_merged(d.merged, WORDS, w - 1u), S, k4);
            const size_t es = rbase + sidx;
            float4 gf = make_float4(0.f, 0.f, 0.f, 0.f);
            float J[SPT];
#pragma unroll
            for (int k = 0; k < SPT; ++k) {
                const float4 cb = d.tape[(es * SPT + k) * 32 + lane];
                const float4 l = lam[k];
                J[k] = l.x * av * (f.x - cb.x) + l.y * av * (f.y - cb.y) + l.z * av * (f.z - cb.z) +
                       l.w * av * (av - cb.w);
                if ((m >> (sub + 8 * k)) & 1u) {
                    gf.x += l.x * av;
                    gf.y += l.y * av;
                    gf.z += l.z * av;
                    gf.w += l.x * (f.x - cb.x) + l.y * (f.y - cb.y) + l.z * (f.z - cb.z) + l.w * (2.f * av - cb.w);
                    lam[k] = make_float4(l.x * om, l.y * om, l.z * om, l.w * om);
                }
            }
            group_adjoint<S>(a, d, d.heads[w - 1], a.fill_rule[path], J, lane);
            gf = warp_sum4(gf, lane);
            if (lane == 0 && (gf.x != 0.f || gf.y != 0.f || gf.z != 0.f || gf.w != 0.f))
                add_fill_grad(d, acc, cache, tag, path, gf);
        }
    }
    if (tag) {  // the warp's cached gradients
        __syncwarp();
        for (int i = lane; i < kDiffCacheSlots; i += 32)
            if (tag[i] != 0xFFFFFFFFu) global_fill_grad(d, tag[i], cache[i]);
    }
    if (acc) {
        __syncthreads();
        for (int i = threadIdx.x; i < a.P; i += kDiffThreads) {
            const float4 v = acc[i];
            if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) {
                atomicAdd(&d.grad_fill[i].x, v.x);
                atomicAdd(&d.grad_fill[i].y, v.y);
                atomicAdd(&d.grad_fill[i].z, v.z);
                atomicAdd(&d.grad_fill[i].w, v.w);
            }
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
    float m[16];
    int Wv = a.W, Hv = a.H;
    if (a.path_scene != nullptr) {
        const SceneInfo *sc = a.scenes + a.path_scene[pid];
#pragma unroll
        for (int k = 0; k < 16; ++k) m[k] = sc->m[k];
        Wv = sc->W;
        Hv = sc->H;
    } else {
#pragma unroll
        for (int k = 0; k < 16; ++k) m[k] = a.m[k];
    }
    float ov[4], dox[4], doy[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        ov[r] = m[4 * r] * xa + m[4 * r + 1] * ya + m[4 * r + 3];
        dox[r] = m[4 * r];
        doy[r] = m[4 * r + 1];
    }
    float q[3], qx[3], qy[3];
    const float i3 = 1.f / ov[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        q[r] = ov[r] * i3;
        qx[r] = (dox[r] - q[r] * dox[3]) * i3;
        qy[r] = (doy[r] - q[r] * doy[3]) * i3;
    }
    const float w = (float)Wv, h = (float)Hv, z = (float)min(Wv, Hv);
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

template <int S, bool BWD, bool CACHE>
void run_diff(const FrameArgs &a, const DiffArgs &d, unsigned grid, size_t smem, cudaStream_t s) {
    if constexpr (BWD || !CACHE) {  // the forward pass accumulates nothing
        cudaFuncSetAttribute(k_diff<S, BWD, CACHE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_diff<S, BWD, CACHE><<<grid, kDiffThreads, smem, s>>>(a, d);
    }
}

template <bool BWD>
int launch_diff(const FrameArgs &a, const DiffArgs &d, cudaStream_t s) {
    if (a.n_bins <= 0) return 0;
    cudaMemsetAsync(d.queue, 0, sizeof(uint32_t), s);
    const unsigned grid = (unsigned)diff_blocks(a);
    int n = 1;
    if (d.npairs > 0) {
        k_diff_gather<<<(unsigned)((d.npairs + 255) / 256), 256, 0, s>>>(d, a.S / 8);
        ++n;
    }
    // backward: block-wide per-path accumulators up to kDiffPathAcc paths,
    // per-warp path caches beyond
    const bool cache = BWD && a.P > kDiffPathAcc;
    const size_t smem = !BWD  ? 0
                        : cache ? (sizeof(float4) + sizeof(uint32_t)) * kDiffCacheSlots * (kDiffThreads / 32)
                                : sizeof(float4) * (size_t)std::max(a.P, 1);
    if (a.S == 8) {
        cache ? run_diff<8, BWD, true>(a, d, grid, smem, s) : run_diff<8, BWD, false>(a, d, grid, smem, s);
    } else if (a.S == 16) {
        cache ? run_diff<16, BWD, true>(a, d, grid, smem, s) : run_diff<16, BWD, false>(a, d, grid, smem, s);
    } else {
        cache ? run_diff<32, BWD, true>(a, d, grid, smem, s) : run_diff<32, BWD, false>(a, d, grid, smem, s);
    }
    if (BWD && d.nf > 0) {
        k_diff_chain<<<(unsigned)((d.nf + 255) / 256), 256, 0, s>>>(a, d);
        ++n;
    }
    return n;
}

}  // namespace

int64_t diff_blocks(const FrameArgs &a) {
    const int64_t units = a.n_bins * (kTileW / 2);
    const int64_t per_block = kDiffThreads / 32;
    return std::max<int64_t>(1, std::min<int64_t>((units + per_block - 1) / per_block, (int64_t)diff_sm_count() * 4));
}

int64_t diff_tape_words(const FrameArgs &a, int depth) {
    return diff_blocks(a) * (int64_t)depth * (a.S / 8) * kDiffThreads;
}

int64_t diff_tape_rec_words(const FrameArgs &a, int depth) {
    return diff_blocks(a) * (int64_t)(kDiffThreads / 32) * depth * 3;
}

__global__ void k_accumulate(float *__restrict__ dst, const float *__restrict__ src, int64_t n, int first) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = first ? src[i] : dst[i] + src[i];
}

int launch_accumulate(float *dst, const float *src, int64_t n, int first, cudaStream_t s) {
    if (n <= 0) return 0;
    k_accumulate<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dst, src, n, first);
    return 1;
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
