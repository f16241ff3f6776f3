// spr_kernels.cu -- the scanline fill pipeline on sm_103a.
//
// Stage map (reference function -> kernel here):
//   k_transformVertex (cu:36-105)                    -> k_transform
//   k_make_intersection_0 + escan (ras_cut.h:1254)   -> k_curve_count + scan
//   k_make_intersection_1 (ras_cut.h:1484)           -> k_curve_emit
//   k_gen_fragment_and_stencil_mask (cu:112-441)     -> k_fragment
//   cuda_seg_sort_int_by_int (cuda_sort.cu:12)       -> radix_sort (spr_sort.cu)
//   k_shuffleFragments + int8 scan (cu:444, 1099)    -> k_wn_reduce / k_wn_down
//   k_mark_merged_fragment_and_span + scans +
//   k_gen_gl_merged_fragment_and_span (cu:462-868)   -> k_flags_reduce / k_flags_down
//   k_gen_stencil_cuda_sm + block boundary (cu:554)  -> k_stencil
//   OpenGL draw + multisample resolve (cu:1312-1433) -> k_item_tiles, k_emit_pairs,
//                                                       radix_sort, k_bin_bounds, k_resolve
// ("cu" = gpu-scanline/src/rasterizer/R_cut_A_mask_comb_scanline/ras_cut_mask_comb_scanline.cu)

#include <cuda_runtime.h>

#include <cstdint>

#include "spr_device.cuh"
#include "spr_internal.h"

namespace spr {

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(int64_t n, int t = kThreads) { return (unsigned)((n + t - 1) / t); }

__device__ __forceinline__ void load_geom(const CurveDesc &d, const float2 *__restrict__ tv, CurveGeom &g) {
    g.type = (int)(d.type & 0xFFu);
    g.w = g.type == kRational ? d.w : 0.f;
    const int n = g.type & 7;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (j < n) {
            float2 v = tv[d.vpos + j];
            g.px[j] = v.x;
            g.py[j] = v.y;
        } else {
            g.px[j] = 0.f;
            g.py[j] = 0.f;
        }
    }
}

// ---------------------------------------------------------- transform --
__global__ void k_transform(FrameArgs a, float2 *__restrict__ tvert, uint32_t *__restrict__ flags) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < a.V;
    uint32_t pid = 0, bit = 0;
    if (valid) {
        float2 p = a.vertex[i];
        pid = a.vertex_pid[i];
        if (a.affine) {
            const float *A = a.affine + 6 * (size_t)pid;
            float x = A[0] * p.x + A[2] * p.y + A[4];
            float y = A[1] * p.x + A[3] * p.y + A[5];
            p = make_float2(x, y);
        }
        const float iv0 = p.x, iv1 = p.y, iv2 = 0.f, iv3 = 1.f;
        float ov[4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
            ov[r] = a.m[4 * r] * iv0 + a.m[4 * r + 1] * iv1 + a.m[4 * r + 2] * iv2 + a.m[4 * r + 3] * iv3;
        ov[0] /= ov[3];
        ov[1] /= ov[3];
        ov[2] /= ov[3];
        const float w = (float)a.W, h = (float)a.H;
        const float z = (float)min(a.W, a.H);
        const float cutoff = -z * 0.5f;
        if (ov[2] < cutoff) ov[2] = cutoff;
        const float w2 = w * .5f, h2 = h * .5f;
        ov[0] = (ov[0] - w2) * z / (ov[2] + z) + w2;
        ov[1] = (ov[1] - h2) * z / (ov[2] + z) + h2;
        const int xf = ov[0] < 0 ? 0 : (ov[0] <= w ? 1 : 2);
        const int yf = ov[1] < 0 ? 0 : (ov[1] <= h ? 1 : 2);
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
        if (floorf(ov[0]) == ov[0]) ov[0] = ov[0] - 1.f / 256.f;
        tvert[i] = make_float2(ov[0], ov[1]);
    }
    // One atomic per distinct path per warp.
    const uint32_t key = valid ? pid : 0xFFFFFFFFu;
    const uint32_t peers = __match_any_sync(0xffffffffu, key);
    const uint32_t agg = __reduce_or_sync(peers, bit);
    if (valid && (threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1)) atomicOr(&flags[pid], agg);
}

// PATH_VISIBLE (ras_define.h:113-127): not entirely on one side of the viewport.
__global__ void k_path_visible(int P, const uint32_t *__restrict__ flags, uint8_t *__restrict__ vis) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const uint32_t f = flags[p];
    vis[p] = ((f & 0xF8u) && (f & 0x6Bu) && (f & 0x1Fu) && (f & 0xD6u)) ? 1 : 0;
}

// ------------------------------------------------------ intersections --
__global__ void k_curve_count(FrameArgs a, const float2 *__restrict__ tv, const uint8_t *__restrict__ vis,
                              uint32_t *__restrict__ counts) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.C) return;
    const CurveDesc d = a.curves[c];
    CurveGeom g;
    load_geom(d, tv, g);
    float q[5];
    const int np = monotonize(g, vis[d.pid] != 0, q);
    float v0x = g.px[0], v0y = g.py[0];
    uint32_t p = 0;
    for (int i = 0; i < np; ++i) {
        const float t1 = q[i];
        const float v1x = curve_coord(g.type, g.w, g.px, t1), v1y = curve_coord(g.type, g.w, g.py, t1);
        const CutRange cr = cut_range(v0x, v0y, v1x, v1y, a.W, a.H);
        p += 1 + cr.nx + cr.ny;
        v0x = v1x;
        v0y = v1y;
    }
    counts[c] = p;
}

// Entries of one curve in t order: each monotone piece emits its start and
// every crossing with a vertical (x = even) or horizontal (y = even) cell
// line, the two crossing chains merged by t; equal t values OR their flags.
__global__ void k_curve_emit(FrameArgs a, const float2 *__restrict__ tv, const uint8_t *__restrict__ vis,
                             const uint32_t *__restrict__ offsets, int2 *__restrict__ entries) {
    const int cid = blockIdx.x * blockDim.x + threadIdx.x;
    if (cid >= a.C) return;
    const CurveDesc d = a.curves[cid];
    CurveGeom g;
    load_geom(d, tv, g);
    float q[5];
    const int np = monotonize(g, vis[d.pid] != 0, q);
    int2 *out = entries + offsets[cid];
    float t0_ms = 0.f;
    float v0x = g.px[0], v0y = g.py[0];
    int p = 0;
    for (int ms = 0; ms < np; ++ms) {
        const float traw = q[ms];
        const float v1x = curve_coord(g.type, g.w, g.px, traw), v1y = curve_coord(g.type, g.w, g.py, traw);
        const uint32_t tb = fbits(traw) & 0xFFFFFFFCu;
        const float t1_ms = (floorf(v1x) == v1x) ? ffrom(tb | 2u) : ffrom(tb | 3u);
        const CutRange cr = cut_range(v0x, v0y, v1x, v1y, a.W, a.H);
        int nx = cr.nx, ny = cr.ny;
        const int n_loop = nx + ny + 1;
        float x = (float)(cr.dx < 0.f ? cr.xe : cr.xb);
        float y = (float)(cr.dy < 0.f ? cr.ye : cr.yb);
        float slot0 = t0_ms, slot1 = t0_ms;
        uint32_t last = fbits(-1.f);
        for (int i = -1; i < n_loop; ++i) {
            float t_solve = 0.f, c = 0.f, t_min;
            int side = 0;
            if (i == -1) {
                t_min = slot0;
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
            } else if (slot0 <= slot1) {
                t_min = slot0;
                side = 0;
                if (nx > 0) {
                    nx--;
                    c = x;
                    x += cr.dx;
                } else {
                    t_solve = 2.f;
                }
            } else {
                t_min = slot1;
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
                uint32_t ob = fbits(t_min);
                if ((ob & 0xFFFFFFFCu) == (last & 0xFFFFFFFCu)) {
                    ob |= last;
                    out[p - 1] = make_int2(cid, (int)ob);
                }
                out[p] = make_int2(cid, (int)ob);
                last = ob;
                p++;
            }
            if (t_solve < 2.f) t_solve = solve_crossing(g, side ? g.py : g.px, c, t_min, t1_ms);
            const float st = ffrom((fbits(t_solve) & 0xFFFFFFFCu) | (uint32_t)side);
            if (side)
                slot1 = st;
            else
                slot0 = st;
        }
        t0_ms = t1_ms;
        v0x = v1x;
        v0y = v1y;
    }
}

// ---------------------------------------------------------- fragments --
template <int S>
__global__ void __launch_bounds__(kThreads) k_fragment(FrameArgs a, const float2 *__restrict__ tv,
                                                       const int2 *__restrict__ entries, int64_t nf,
                                                       int32_t *__restrict__ key_out, uint32_t *__restrict__ pid_out,
                                                       int8_t *__restrict__ wn_out, uint32_t *__restrict__ mask_out,
                                                       uint64_t *__restrict__ sort_key, uint32_t *__restrict__ sort_val) {
    constexpr int WORDS = S / 8;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    const int2 e0 = entries[i];
    const int2 e1 = (i + 1) != nf ? entries[i + 1] : make_int2(-1, 0x3f800000);
    int f0 = e0.y & 1, f1 = e1.y & 1;
    float t0 = ffrom((uint32_t)e0.y & 0xFFFFFFFCu);
    float t1 = ffrom((uint32_t)e1.y & 0xFFFFFFFCu);
    if (t0 < 0) t0 = 0.f;
    if (t1 < 0) t1 = 0.f;
    if (t0 == 0.f || t0 == 1.f) f0 = 1;
    if (t1 == 0.f || t1 == 1.f) f1 = 1;
    const int cid = e0.x;
    const CurveDesc d = a.curves[cid];
    const uint32_t pathid = d.pid;
    int32_t yx = kInvalidKey;
    if (e0.x != e1.x) t1 = 1.f;
    int wnchg = 0, swn = 0;
    uint32_t mask[4] = {0u, 0u, 0u, 0u};
    if (t0 < t1) {
        CurveGeom g;
        load_geom(d, tv, g);
        const float fi0 = 0 / 1.f, fi1 = 1 / 1.f;
        const float ta = (1 - fi0) * t0 + fi0 * t1;
        const float tb = (1 - fi1) * t0 + fi1 * t1;
        const float c0x = curve_coord(g.type, g.w, g.px, ta), c0y = curve_coord(g.type, g.w, g.py, ta);
        const float c1x = curve_coord(g.type, g.w, g.px, tb), c1y = curve_coord(g.type, g.w, g.py, tb);
        const bool rev = ((d.type >> 8) & 1u) != 0;
        const float vfx = rev ? c1x : c0x, vfy = rev ? c1y : c0y;
        const float vlx = rev ? c0x : c1x, vly = rev ? c0y : c1y;
        const int sf = rev ? f1 : f0;
        const int sl = rev ? f0 : f1;
        const int rx = floor2((vfx + vlx) * 0.5f);
        const int ry = floor2((vfy + vly) * 0.5f);
        const int px = min(max(rx, -2), (int)(((uint32_t)a.W & 0xFFFFFFFEu) + 2));
        const int py = min(max(ry, -2), (int)(((uint32_t)a.H & 0xFFFFFFFEu) + 2));
        const uint32_t ys = (uint32_t)(py + 0x7FFF) << 16;
        const uint32_t xs = (uint32_t)(px + 0x7FFF) & 0xFFFFu;
        if ((uint32_t)ry < (uint32_t)a.H) yx = (int32_t)(ys | xs);
        const int wy = py + 1;
        if (vfy == vly) {
            swn = 0;
        } else if (vfy <= wy && wy < vly) {
            swn = -1;
        } else if (vly <= wy && wy < vfy) {
            swn = 1;
        }
        if (vfy < vly) {
            wnchg = -1;
        } else if (vfy > vly) {
            wnchg = 1;
        } else {
            wnchg = (vfx < vlx) ? 1 : -1;
        }
        float lx = 0.f, ly = 0.f, rgt_y = 0.f;
        int left_flag = 1;
        if (vfx < vlx) {
            lx = vfx;
            ly = vfy;
            rgt_y = vly;
            left_flag = sf;
        } else if (vfx > vlx) {
            lx = vlx;
            ly = vly;
            rgt_y = vfy;
            left_flag = sl;
        } else if (vfx < px + 1) {
            if (sf == 0) {
                lx = vfx;
                ly = vfy;
                rgt_y = vly;
                left_flag = 0;
            } else if (sl == 0) {
                lx = vlx;
                ly = vly;
                rgt_y = vfy;
                left_flag = 0;
            }
        }
        (void)lx;
        uint32_t lm[4] = {0u, 0u, 0u, 0u};
        if (left_flag == 0) {
            vertical_mask<S>((ly - py) * .5f, lm);
            if (ly <= py + 1) {
                if (ly >= rgt_y) wnchg = -wnchg;
            } else {
                if (ly < rgt_y) wnchg = -wnchg;
#pragma unroll
                for (int w = 0; w < 4; ++w) lm[w] = ~lm[w];
            }
        }
        const float bx = (float)px, by = (float)py;
        const float q0x = (c0x - bx) * .5f, q0y = (c0y - by) * .5f;
        const float q1x = (c1x - bx) * .5f, q1y = (c1y - by) * .5f;
        uint32_t vm[4];
        vertical_mask2<S>(q0y, q1y, vm);
        const int texel = table_texel(q0x, q0y, q1x, q1y);
        if (S == 8) {
            const uint32_t tm = __ldg(a.mask_table + texel);
            mask[0] = (tm & vm[0]) ^ lm[0];
        } else {
            const uint4 tm = __ldg(reinterpret_cast<const uint4 *>(a.mask_table) + texel);
            mask[0] = (tm.x & vm[0]) ^ lm[0];
            mask[1] = (tm.y & vm[1]) ^ lm[1];
            mask[2] = (tm.z & vm[2]) ^ lm[2];
            mask[3] = (tm.w & vm[3]) ^ lm[3];
        }
    }
    key_out[i] = yx;
    pid_out[i] = pathid | ((uint32_t)wnchg << 30);
    wn_out[i] = (int8_t)swn;
    if (WORDS == 1) {
        mask_out[i] = mask[0];
    } else {
        reinterpret_cast<uint4 *>(mask_out)[i] = make_uint4(mask[0], mask[1], mask[2], mask[3]);
    }
    const int nrows = (a.H + 1) / 2;
    sort_key[i] = ((uint64_t)pathid << 24) | (uint64_t)local_sort_key(yx, nrows);
    sort_val[i] = (uint32_t)i;
}

// --------------------------------------------- winding scan + marks --
constexpr int kFlagThreads = 256;
constexpr int kFlagItems = 8;
constexpr int kFlagTile = kFlagThreads * kFlagItems;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += n;
    }
    return v;
}
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *sw, uint32_t *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int W = kFlagThreads / 32;
    uint32_t inc = warp_incl_scan(v);
    if (lane == 31) sw[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = lane < W ? sw[lane] : 0u;
        uint32_t ti = warp_incl_scan(t);
        if (lane < W) sw[lane] = ti - t;
        if (lane == W - 1) sw[W] = ti;
    }
    __syncthreads();
    uint32_t r = sw[warp] + inc - v;
    *total = sw[W];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kFlagThreads) k_wn_reduce(int64_t nf, const uint32_t *__restrict__ perm,
                                                            const int8_t *__restrict__ wn, uint32_t *__restrict__ sums) {
    __shared__ uint32_t sw[kFlagThreads / 32 + 1];
    const int64_t base = (int64_t)blockIdx.x * kFlagTile + (int64_t)threadIdx.x * kFlagItems;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kFlagItems; ++k) {
        const int64_t i = base + k;
        if (i < nf) s += (uint32_t)(int32_t)wn[perm[i]];
    }
    uint32_t total;
    block_excl_scan(s, sw, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kFlagThreads) k_wn_down(int64_t nf, const uint32_t *__restrict__ perm,
                                                          const int8_t *__restrict__ wn,
                                                          const uint32_t *__restrict__ sums,
                                                          int8_t *__restrict__ wn_scan) {
    __shared__ uint32_t sw[kFlagThreads / 32 + 1];
    const int64_t base = (int64_t)blockIdx.x * kFlagTile + (int64_t)threadIdx.x * kFlagItems;
    uint32_t v[kFlagItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kFlagItems; ++k) {
        const int64_t i = base + k;
        v[k] = i < nf ? (uint32_t)(int32_t)wn[perm[i]] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t p = block_excl_scan(s, sw, &total) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kFlagItems; ++k) {
        const int64_t i = base + k;
        if (i < nf) wn_scan[i] = (int8_t)(uint8_t)p;
        p += v[k];
    }
}

struct Mark {
    uint32_t ff, sf;
};

// k_mark_merged_fragment_and_span (cu:462-535) on sorted position i.
__device__ __forceinline__ Mark mark_at(int64_t i, const uint64_t *__restrict__ skey, const int8_t *__restrict__ wn_scan,
                                        const uint8_t *__restrict__ rule, int W, int H, int nrows) {
    const uint64_t k1 = skey[i];
    const uint32_t key1 = (uint32_t)key_from_local((uint32_t)(k1 & 0xFFFFFFu), nrows);
    const int x1 = key_x(key1), y1 = key_y(key1);
    const bool oob = x1 < 0 || y1 < 0 || x1 >= W || y1 >= H;
    Mark m{0u, 0u};
    if (i == 0) {
        m.ff = oob ? 0u : 1u;
        return m;
    }
    const uint64_t k0 = skey[i - 1];
    const uint32_t p0 = (uint32_t)(k0 >> 24), p1 = (uint32_t)(k1 >> 24);
    const uint32_t key0 = (uint32_t)key_from_local((uint32_t)(k0 & 0xFFFFFFu), nrows);
    const int x0 = key_x(key0), y0 = key_y(key0);
    m.ff = oob ? 0u : ((p0 != p1 || key0 != key1) ? 1u : 0u);
    const uint8_t fr = rule[p1];
    const int8_t w = wn_scan[i];
    const bool wf = (fr == 0 && w != 0) || (fr == 1 && (w & 1));
    m.sf = (y0 == y1 && (x0 + 2) < x1 && p0 == p1 && wf) ? 1u : 0u;
    return m;
}

__global__ void __launch_bounds__(kFlagThreads) k_flags_reduce(FrameArgs a, int64_t nf, const uint64_t *__restrict__ skey,
                                                               const int8_t *__restrict__ wn_scan,
                                                               uint32_t *__restrict__ fsum, uint32_t *__restrict__ ssum) {
    __shared__ uint32_t sw[kFlagThreads / 32 + 1];
    const int nrows = (a.H + 1) / 2;
    const int64_t base = (int64_t)blockIdx.x * kFlagTile + (int64_t)threadIdx.x * kFlagItems;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kFlagItems; ++k) {
        const int64_t i = base + k;
        if (i < nf) {
            const Mark m = mark_at(i, skey, wn_scan, a.fill_rule, a.W, a.H, nrows);
            s += m.ff | (m.sf << 16);
        }
    }
    uint32_t total;
    block_excl_scan(s, sw, &total);
    if (threadIdx.x == 0) {
        fsum[blockIdx.x] = total & 0xFFFFu;
        ssum[blockIdx.x] = total >> 16;
    }
}

__global__ void __launch_bounds__(kFlagThreads) k_flags_down(FrameArgs a, int64_t nf, int64_t ntiles,
                                                             const uint64_t *__restrict__ skey,
                                                             const int8_t *__restrict__ wn_scan,
                                                             const uint32_t *__restrict__ fsum,
                                                             const uint32_t *__restrict__ ssum, int4 *__restrict__ draw,
                                                             uint32_t *__restrict__ heads,
                                                             FrameCounters *__restrict__ counters) {
    __shared__ uint32_t sw[kFlagThreads / 32 + 1];
    const int nrows = (a.H + 1) / 2;
    const int64_t base = (int64_t)blockIdx.x * kFlagTile + (int64_t)threadIdx.x * kFlagItems;
    Mark mk[kFlagItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kFlagItems; ++k) {
        const int64_t i = base + k;
        mk[k] = i < nf ? mark_at(i, skey, wn_scan, a.fill_rule, a.W, a.H, nrows) : Mark{0u, 0u};
        s += mk[k].ff | (mk[k].sf << 16);
    }
    uint32_t total;
    const uint32_t pre = block_excl_scan(s, sw, &total);
    uint32_t nfb = fsum[blockIdx.x] + (pre & 0xFFFFu);
    uint32_t nsb = ssum[blockIdx.x] + (pre >> 16);
#pragma unroll
    for (int k = 0; k < kFlagItems; ++k) {
        const int64_t i = base + k;
        if (i >= nf) break;
        const uint32_t ff = mk[k].ff, sf = mk[k].sf;
        if (ff | sf) {
            const uint64_t k1 = skey[i];
            const uint32_t p = (uint32_t)(k1 >> 24);
            const int32_t fill = (int32_t)a.fill_rgba[p];
            const uint32_t key1 = (uint32_t)key_from_local((uint32_t)(k1 & 0xFFFFFFu), nrows);
            if (ff) {
                const int32_t pos = (int32_t)(((uint32_t)key_y(key1) << 16) | (uint32_t)key_x(key1));
                draw[nfb + nsb] = make_int4(pos, 2, fill, (int)(nfb + 1));
                heads[nfb] = (uint32_t)i;
            }
            if (sf) {
                const uint32_t key0 = (uint32_t)key_from_local((uint32_t)(skey[i - 1] & 0xFFFFFFu), nrows);
                const int y0 = key_y(key0);
                int x0 = (int16_t)(key_x(key0) + 2);
                const int x1 = key_x(key1);
                x0 = max(0, x0);
                const int32_t pos = (int32_t)(((uint32_t)y0 << 16) | (uint32_t)x0);
                draw[nfb + nsb + ff] = make_int4(pos, x1 - x0, fill, 0);
            }
        }
        nfb += ff;
        nsb += sf;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        counters->n_merged = fsum[ntiles];
        counters->n_span = ssum[ntiles];
    }
}

// ------------------------------------------------------- merged masks --
// Per merged fragment: the scanned winding number plus the signed boundary
// masks of every fragment of the (path, cell) group, in 8-bit lanes per
// mask bit (the reference's packed counters), reduced to the 7-bit winding
// number and tested against the fill rule.
template <int S>
__global__ void __launch_bounds__(kThreads) k_stencil(FrameArgs a, int64_t nf, int64_t nm,
                                                      const uint64_t *__restrict__ skey,
                                                      const uint32_t *__restrict__ perm,
                                                      const uint32_t *__restrict__ pidw,
                                                      const uint32_t *__restrict__ mask,
                                                      const int8_t *__restrict__ wn_scan,
                                                      const uint32_t *__restrict__ heads,
                                                      uint32_t *__restrict__ merged) {
    constexpr int WORDS = S / 8;
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nm) return;
    const int64_t h = heads[g];
    const uint64_t kh = skey[h];
    const int32_t w0 = wn_scan[h];
    const uint32_t init = 0x01010101u * (uint32_t)w0;
    uint32_t acc[WORDS][8];
#pragma unroll
    for (int w = 0; w < WORDS; ++w)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[w][b] = init;
    for (int64_t j = h; j < nf && skey[j] == kh; ++j) {
        const uint32_t raw = perm[j];
        const int32_t chg = (int32_t)pidw[raw] >> 30;
        if (chg == 0) continue;
        uint32_t m[WORDS];
        if constexpr (WORDS == 1) {
            m[0] = mask[raw];
        } else {
            const uint4 v = reinterpret_cast<const uint4 *>(mask)[raw];
            m[0] = v.x;
            m[1] = v.y;
            m[2] = v.z;
            m[3] = v.w;
        }
#pragma unroll
        for (int w = 0; w < WORDS; ++w)
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                const uint32_t bits = (m[w] >> b) & 0x01010101u;
                acc[w][b] = chg > 0 ? acc[w][b] + bits : acc[w][b] - bits;
            }
    }
    const int fr = a.fill_rule[(uint32_t)(kh >> 24)];
#pragma unroll
    for (int w = 0; w < WORDS; ++w) {
        uint32_t ret = 0;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            uint32_t wv = (0x80808080u + acc[w][b]) & 0x7f7f7f7fu;
            if (fr == 0) {
                wv |= wv >> 4;
                wv |= wv >> 2;
                wv |= wv >> 1;
            }
            ret |= (wv & 0x01010101u) << b;
        }
        merged[g * WORDS + w] = ret;
    }
}

// ------------------------------------------------------------ resolve --
constexpr int kTileW = 32;  // pixel columns per resolve bin (one warp)
constexpr int kResolveWarps = 8;

__device__ __forceinline__ void item_cols(const int4 &it, int W, int &x0, int &x1) {
    const int x = (int)((uint32_t)it.x & 0xFFFFu);
    x0 = max(x, 0);
    x1 = min(x + it.y, W);
}

__global__ void k_item_tiles(FrameArgs a, const int4 *__restrict__ draw, int64_t n, uint32_t *__restrict__ cnt) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int x0, x1;
    item_cols(draw[i], a.W, x0, x1);
    cnt[i] = x1 > x0 ? (uint32_t)((x1 - 1) / kTileW - x0 / kTileW + 1) : 0u;
}

__global__ void k_emit_pairs(FrameArgs a, const int4 *__restrict__ draw, int64_t n, const uint32_t *__restrict__ offs,
                             uint32_t *__restrict__ pkey, uint32_t *__restrict__ pval) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int4 it = draw[i];
    int x0, x1;
    item_cols(it, a.W, x0, x1);
    if (x1 <= x0) return;
    const int ntx = (a.W + kTileW - 1) / kTileW;
    const int row = (it.x >> 16) / 2;
    uint32_t o = offs[i];
    for (int t = x0 / kTileW; t <= (x1 - 1) / kTileW; ++t) {
        pkey[o] = (uint32_t)(row * ntx + t);
        pval[o] = (uint32_t)i;
        ++o;
    }
}

__global__ void k_bin_bounds(const uint32_t *__restrict__ key, int64_t n, uint32_t *__restrict__ start,
                             uint32_t *__restrict__ end) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = key[i];
    if (i == 0 || key[i - 1] != k) start[k] = (uint32_t)i;
    if (i == n - 1 || key[i + 1] != k) end[k] = (uint32_t)(i + 1);
}

struct SmemTables {
    float dec[256];
    float lin[256];
    float th[256];
    uint8_t bin[4096];
};

__device__ __forceinline__ uint32_t enc_lin(float v) {
    const float c = fmin_r(fmax_r(v, 0.f), 1.f);
    return (uint32_t)cvt_rzi(c * 255.f + 0.5f);
}
__device__ __forceinline__ uint32_t enc_srgb(const SmemTables &t, float v) {
    const float c = fmin_r(fmax_r(v, 0.f), 1.f);
    const int b = min(cvt_rzi(c * 4096.f), 4095);
    uint32_t k = t.bin[b];
    if (k < 255 && c >= t.th[k]) ++k;
    return k;
}

template <bool SRGB>
__device__ __forceinline__ uint32_t blend_sample(const SmemTables &t, uint32_t dv, float sr, float sg, float sb, float a,
                                                 float om) {
    const float dr = t.dec[dv & 0xFF], dg = t.dec[(dv >> 8) & 0xFF], db = t.dec[(dv >> 16) & 0xFF];
    const float da = t.lin[dv >> 24];
    const float orr = sr * a + dr * om;
    const float og = sg * a + dg * om;
    const float ob = sb * a + db * om;
    const float oa = a * a + da * om;
    uint32_t er, eg, eb;
    if (SRGB) {
        er = enc_srgb(t, orr);
        eg = enc_srgb(t, og);
        eb = enc_srgb(t, ob);
    } else {
        er = enc_lin(orr);
        eg = enc_lin(og);
        eb = enc_lin(ob);
    }
    return er | (eg << 8) | (eb << 16) | (enc_lin(oa) << 24);
}

// One warp per bin of (cell row, 32 pixel columns); lane = pixel column,
// two pixel rows each.  Items of the bin are applied in draw-list order to
// the per-sample RGBA8 state kept in shared memory, then every pixel is
// averaged over its samples.
template <int S, bool MS, bool SRGB>
__global__ void __launch_bounds__(kResolveWarps * 32) k_resolve(FrameArgs a, const int4 *__restrict__ draw,
                                                                 const uint32_t *__restrict__ merged,
                                                                 const uint32_t *__restrict__ pval,
                                                                 const uint32_t *__restrict__ bstart,
                                                                 const uint32_t *__restrict__ bend,
                                                                 uint32_t *__restrict__ image) {
    constexpr int SPP = MS ? S : 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemTables &T = *reinterpret_cast<SmemTables *>(smem_raw);
    int4 *stage = reinterpret_cast<int4 *>(smem_raw + sizeof(SmemTables));
    uint32_t *state = reinterpret_cast<uint32_t *>(smem_raw + sizeof(SmemTables) + kResolveWarps * 32 * sizeof(int4));
    {
        const ResolveTables *rt = a.rtables;
        for (int i = threadIdx.x; i < 256; i += blockDim.x) {
            T.dec[i] = SRGB ? rt->srgb_dec[i] : rt->lin_dec[i];
            T.lin[i] = rt->lin_dec[i];
            T.th[i] = rt->threshold[i];
        }
        for (int i = threadIdx.x; i < 4096; i += blockDim.x) T.bin[i] = rt->bin[i];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ntx = (a.W + kTileW - 1) / kTileW;
    const int nrows = (a.H + 1) / 2;
    const int64_t b = (int64_t)blockIdx.x * kResolveWarps + warp;
    if (b >= (int64_t)ntx * nrows) return;
    const int row = (int)(b / ntx), tile = (int)(b % ntx);
    const int px = tile * kTileW + lane;
    const int y0 = row * 2;
    int4 *st = stage + warp * 32;
    uint32_t *ws = state + warp * 2 * SPP * 32;
#pragma unroll
    for (int py = 0; py < 2; ++py)
        for (int s = 0; s < SPP; ++s) ws[(py * SPP + s) * 32 + lane] = 0xFFFFFFFFu;
    const uint32_t beg = bstart[b], fin = bend[b];
    const float *dec = T.dec;
    for (uint32_t base = beg; base < fin; base += 32) {
        if (base + lane < fin) st[lane] = draw[pval[base + lane]];
        __syncwarp();
        const int cnt = (int)min(32u, fin - base);
        for (int q = 0; q < cnt; ++q) {
            const int4 it = st[q];
            const int x = (int)((uint32_t)it.x & 0xFFFFu);
            if (px < x || px >= x + it.y || px >= a.W) continue;
            const uint32_t c = (uint32_t)it.z;
            const float sr = dec[c & 0xFF], sg = dec[(c >> 8) & 0xFF], sb = dec[(c >> 16) & 0xFF];
            const float sa = T.lin[c >> 24];
#pragma unroll
            for (int py = 0; py < 2; ++py) {
                if (y0 + py >= a.H) continue;
                uint32_t m = 0xFFFFFFFFu;
                if (it.w != 0) {
                    const int k = (px - x) * 2 + py;
                    if (S == 8)
                        m = (__ldg(merged + (it.w - 1)) >> (8 * k)) & 0xFFu;
                    else
                        m = __ldg(merged + (int64_t)(it.w - 1) * 4 + k);
                }
                uint32_t *pst = ws + py * SPP * 32 + lane;
                if (MS) {
                    if (S == 8) m &= 0xFFu;
                    const float om = 1.f - sa;
                    while (m) {
                        const int s = __ffs(m) - 1;
                        m &= m - 1;
                        pst[s * 32] = blend_sample<SRGB>(T, pst[s * 32], sr, sg, sb, sa, om);
                    }
                } else {
                    const int cntb = __popc(S == 8 ? (m & 0xFFu) : m);
                    const float aa = sa * ((float)cntb / (float)S);
                    pst[0] = blend_sample<SRGB>(T, pst[0], sr, sg, sb, aa, 1.f - aa);
                }
            }
        }
        __syncwarp();
    }
    if (px >= a.W) return;
#pragma unroll
    for (int py = 0; py < 2; ++py) {
        const int yy = y0 + py;
        if (yy >= a.H) continue;
        const uint32_t *pst = ws + py * SPP * 32 + lane;
        float ar = 0.f, ag = 0.f, ab = 0.f, aa = 0.f;
        for (int s = 0; s < SPP; ++s) {
            const uint32_t v = pst[s * 32];
            ar += dec[v & 0xFF];
            ag += dec[(v >> 8) & 0xFF];
            ab += dec[(v >> 16) & 0xFF];
            aa += T.lin[v >> 24];
        }
        const float n = (float)SPP;
        ar /= n;
        ag /= n;
        ab /= n;
        aa /= n;
        uint32_t out;
        if (SRGB)
            out = enc_srgb(T, ar) | (enc_srgb(T, ag) << 8) | (enc_srgb(T, ab) << 16) | (enc_lin(aa) << 24);
        else
            out = enc_lin(ar) | (enc_lin(ag) << 8) | (enc_lin(ab) << 16) | (enc_lin(aa) << 24);
        image[(int64_t)yy * a.W + px] = out;
    }
}

__global__ void k_fill(uint32_t *image, int64_t n, uint32_t v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) image[i] = v;
}

__global__ void k_decode_keys(const uint64_t *__restrict__ skey, int64_t n, int nrows, int32_t *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = key_from_local((uint32_t)(skey[i] & 0xFFFFFFu), nrows);
}

template <int S, bool MS, bool SRGB>
void resolve_variant(const FrameArgs &a, const int4 *draw, const uint32_t *merged, const uint32_t *pval,
                     const uint32_t *bstart, const uint32_t *bend, uint32_t *image, cudaStream_t s) {
    constexpr int SPP = MS ? S : 1;
    const size_t smem = sizeof(SmemTables) + kResolveWarps * 32 * sizeof(int4) +
                        (size_t)kResolveWarps * 2 * SPP * 32 * sizeof(uint32_t);
    cudaFuncSetAttribute(k_resolve<S, MS, SRGB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int64_t nbins = (int64_t)((a.W + kTileW - 1) / kTileW) * ((a.H + 1) / 2);
    k_resolve<S, MS, SRGB><<<grid_for(nbins, kResolveWarps), kResolveWarps * 32, smem, s>>>(a, draw, merged, pval,
                                                                                           bstart, bend, image);
}

}  // namespace

void launch_transform(const FrameArgs &a, float2 *tvert, uint32_t *path_flags, uint8_t *path_visible, cudaStream_t s) {
    cudaMemsetAsync(path_flags, 0, sizeof(uint32_t) * (size_t)a.P, s);
    if (a.V > 0) k_transform<<<grid_for(a.V), kThreads, 0, s>>>(a, tvert, path_flags);
    if (a.P > 0) k_path_visible<<<grid_for(a.P), kThreads, 0, s>>>(a.P, path_flags, path_visible);
}

void launch_curve_count(const FrameArgs &a, const float2 *tvert, const uint8_t *vis, uint32_t *counts, cudaStream_t s) {
    if (a.C > 0) k_curve_count<<<grid_for(a.C), kThreads, 0, s>>>(a, tvert, vis, counts);
}

void launch_curve_emit(const FrameArgs &a, const float2 *tvert, const uint8_t *vis, const uint32_t *offsets,
                       int2 *entries, cudaStream_t s) {
    if (a.C > 0) k_curve_emit<<<grid_for(a.C), kThreads, 0, s>>>(a, tvert, vis, offsets, entries);
}

void launch_fragment(const FrameArgs &a, const float2 *tvert, const int2 *entries, int64_t nf, int32_t *key,
                     uint32_t *pidw, int8_t *wn, uint32_t *mask, uint64_t *sort_key, uint32_t *sort_val,
                     cudaStream_t s) {
    if (nf <= 0) return;
    if (a.S == 8)
        k_fragment<8><<<grid_for(nf), kThreads, 0, s>>>(a, tvert, entries, nf, key, pidw, wn, mask, sort_key, sort_val);
    else
        k_fragment<32><<<grid_for(nf), kThreads, 0, s>>>(a, tvert, entries, nf, key, pidw, wn, mask, sort_key, sort_val);
}

int64_t flags_tmp_words(int64_t nf) { return 2 * ((nf + kFlagTile - 1) / kFlagTile + 2); }

void launch_scan_mark(const FrameArgs &a, int64_t nf, const uint64_t *skey, const uint32_t *perm, const int8_t *wn,
                      int8_t *wn_scan, int4 *draw, uint32_t *heads, FrameCounters *counters, uint32_t *tmp,
                      cudaStream_t s) {
    const int64_t ntiles = (nf + kFlagTile - 1) / kFlagTile;
    uint32_t *s0 = tmp, *s1 = tmp + (ntiles + 2);
    k_wn_reduce<<<(unsigned)ntiles, kFlagThreads, 0, s>>>(nf, perm, wn, s0);
    scan_tiles_inplace(s0, ntiles, s);
    k_wn_down<<<(unsigned)ntiles, kFlagThreads, 0, s>>>(nf, perm, wn, s0, wn_scan);
    k_flags_reduce<<<(unsigned)ntiles, kFlagThreads, 0, s>>>(a, nf, skey, wn_scan, s0, s1);
    scan_tiles_inplace(s0, ntiles, s);
    scan_tiles_inplace(s1, ntiles, s);
    k_flags_down<<<(unsigned)ntiles, kFlagThreads, 0, s>>>(a, nf, ntiles, skey, wn_scan, s0, s1, draw, heads, counters);
}

void launch_stencil(const FrameArgs &a, int64_t nf, int64_t nm, const uint64_t *skey, const uint32_t *perm,
                    const uint32_t *pidw, const uint32_t *mask, const int8_t *wn_scan, const uint32_t *heads,
                    uint32_t *merged, cudaStream_t s) {
    if (nm <= 0) return;
    if (a.S == 8)
        k_stencil<8><<<grid_for(nm), kThreads, 0, s>>>(a, nf, nm, skey, perm, pidw, mask, wn_scan, heads, merged);
    else
        k_stencil<32><<<grid_for(nm), kThreads, 0, s>>>(a, nf, nm, skey, perm, pidw, mask, wn_scan, heads, merged);
}

void launch_item_tiles(const FrameArgs &a, const int4 *draw, int64_t n, uint32_t *cnt, cudaStream_t s) {
    if (n > 0) k_item_tiles<<<grid_for(n), kThreads, 0, s>>>(a, draw, n, cnt);
}

void launch_emit_pairs(const FrameArgs &a, const int4 *draw, int64_t n, const uint32_t *offs, uint32_t *pkey,
                       uint32_t *pval, cudaStream_t s) {
    if (n > 0) k_emit_pairs<<<grid_for(n), kThreads, 0, s>>>(a, draw, n, offs, pkey, pval);
}

void launch_bin_bounds(const uint32_t *key, int64_t n, uint32_t *start, uint32_t *end, cudaStream_t s) {
    if (n > 0) k_bin_bounds<<<grid_for(n), kThreads, 0, s>>>(key, n, start, end);
}

void launch_resolve(const FrameArgs &a, const int4 *draw, const uint32_t *merged, const uint32_t *pval,
                    const uint32_t *bstart, const uint32_t *bend, uint32_t *image, cudaStream_t s) {
    const bool ms = a.ms_output != 0, srgb = a.srgb != 0;
    if (a.S == 8) {
        if (ms && srgb) resolve_variant<8, true, true>(a, draw, merged, pval, bstart, bend, image, s);
        else if (ms) resolve_variant<8, true, false>(a, draw, merged, pval, bstart, bend, image, s);
        else if (srgb) resolve_variant<8, false, true>(a, draw, merged, pval, bstart, bend, image, s);
        else resolve_variant<8, false, false>(a, draw, merged, pval, bstart, bend, image, s);
    } else {
        if (ms && srgb) resolve_variant<32, true, true>(a, draw, merged, pval, bstart, bend, image, s);
        else if (ms) resolve_variant<32, true, false>(a, draw, merged, pval, bstart, bend, image, s);
        else if (srgb) resolve_variant<32, false, true>(a, draw, merged, pval, bstart, bend, image, s);
        else resolve_variant<32, false, false>(a, draw, merged, pval, bstart, bend, image, s);
    }
}

void launch_fill(uint32_t *image, int64_t n, uint32_t value, cudaStream_t s) {
    if (n > 0) k_fill<<<grid_for(n), kThreads, 0, s>>>(image, n, value);
}

void launch_decode_keys(const uint64_t *skey, int64_t n, int nrows, int32_t *out, cudaStream_t s) {
    if (n > 0) k_decode_keys<<<grid_for(n), kThreads, 0, s>>>(skey, n, nrows, out);
}

}  // namespace spr
