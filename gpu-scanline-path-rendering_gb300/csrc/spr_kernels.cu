// spr_kernels.cu -- the scanline fill pipeline on sm_103a.
//
// Stage map (reference function -> kernel here):
//   k_transformVertex (cu:36-105)                    -> k_transform
//   k_make_intersection_0 + escan (ras_cut.h:1254)   -> k_curve_count + scan
//   k_make_intersection_1 (ras_cut.h:1484)           -> k_curve_emit
//   k_gen_fragment_and_stencil_mask (cu:112-441)     -> k_fragment
//   cuda_seg_sort_int_by_int (cuda_sort.cu:12)       -> k_segment_sort(_small), radix_sort
//                                                       (spr_sort.cu)
//   k_shuffleFragments + int8 scan (cu:444, 1099),
//   k_mark_merged_fragment_and_span + scans,
//   k_gen_gl_merged_fragment_and_span (cu:444-868)   -> k_scan_mark (one look-back pass)
//   k_gen_stencil_cuda_sm + block boundary (cu:554)  -> k_stencil
//   OpenGL draw + multisample resolve (cu:1312-1433) -> bin counts (k_scan_mark),
//                                                       k_scan_lb, k_bin_scatter,
//                                                       k_bin_sort, k_resolve
// ("cu" = gpu-scanline/src/rasterizer/R_cut_A_mask_comb_scanline/ras_cut_mask_comb_scanline.cu)

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "spr_device.cuh"
#include "spr_internal.h"
#include "spr_lookback.cuh"

namespace spr {

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(int64_t n, int t = kThreads) { return (unsigned)((n + t - 1) / t); }

// Viewport of the scene that path pid belongs to.
struct Dim {
    int W, H;
};
__device__ __forceinline__ Dim dim_of(const FrameArgs &a, uint32_t pid) {
    if (a.path_scene == nullptr) return Dim{a.W, a.H};
    const SceneInfo *sc = a.scenes + __ldg(a.path_scene + pid);
    return Dim{sc->W, sc->H};
}

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
        float m[16];
        int W = a.W, H = a.H;
        if (a.path_scene != nullptr) {
            const SceneInfo *sc = a.scenes + a.path_scene[pid];
#pragma unroll
            for (int k = 0; k < 16; ++k) m[k] = sc->m[k];
            W = sc->W;
            H = sc->H;
        } else {
#pragma unroll
            for (int k = 0; k < 16; ++k) m[k] = a.m[k];
        }
        float ov[4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
            ov[r] = m[4 * r] * iv0 + m[4 * r + 1] * iv1 + m[4 * r + 2] * iv2 + m[4 * r + 3] * iv3;
        ov[0] /= ov[3];
        ov[1] /= ov[3];
        ov[2] /= ov[3];
        const float w = (float)W, h = (float)H;
        const float z = (float)min(W, H);
        const float cutoff = -z * 0.5f;
        if (ov[2] < cutoff) ov[2] = cutoff;
        const float w2 = w * .5f, h2 = h * .5f;
        ov[0] = (ov[0] - w2) * z / (ov[2] + z) + w2;
        ov[1] = (ov[1] - h2) * z / (ov[2] + z) + h2;
        if (a.pass_dy != 0.f) ov[1] = ov[1] - a.pass_dy;
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
    const int np = monotonize_r(g, vis[d.pid] != 0, q);
    const Dim dm = dim_of(a, d.pid);
    float v0x = g.px[0], v0y = g.py[0];
    uint32_t p = 0;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        if (i >= np) break;
        const float t1 = q[i];
        const float v1x = curve_coord(g.type, g.w, g.px, t1), v1y = curve_coord(g.type, g.w, g.py, t1);
        const CutRange cr = cut_range(v0x, v0y, v1x, v1y, dm.W, dm.H);
        p += 1 + cr.nx + cr.ny;
        v0x = v1x;
        v0y = v1y;
    }
    counts[c] = p;
}

// Entries of one curve in t order: each monotone piece emits its start and
// every crossing with a vertical (x = even) or horizontal (y = even) cell
// line, the two crossing chains merged by t; equal t values OR their flags.
// Emission order: curves grouped by type (cubics, whose crossings are
// bisections, first) and within a type by decreasing entry count, so that
// the curves of a warp run the same solver the same number of times and
// the longest start first.  16-bit key, ascending.
__global__ void k_emit_keys(FrameArgs a, const uint32_t *__restrict__ counts, uint32_t *__restrict__ key,
                            uint32_t *__restrict__ val) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.C) return;
    const uint32_t type = a.curves[c].type & 0xFFu;
    const uint32_t rank = type == (uint32_t)kCubic ? 0u : (type == (uint32_t)kRational ? 1u : (type == (uint32_t)kQuad ? 2u : 3u));
    key[c] = (rank << 13) | (0x1FFFu - min(counts[c], 0x1FFFu));
    val[c] = (uint32_t)c;
}

// Entries of one monotone piece, whose chain starts from the piece's own
// t0 and is solved crossing by crossing (k_make_intersection_impl_1,
// ras_cut.h:837-1241): every piece is an independent work item.
struct PieceState {
    CurveGeom g;
    int2 *out;
    int cid, p, i, n_loop, nx, ny;
    float x, y, dx, dy, slot0, slot1, t1_ms;
    uint32_t last;
};

// Sets up piece ms of a curve (v0, v1: its end points; t0_ms: the previous
// piece's end parameter with its flags, 0 for the first).
__device__ __forceinline__ void piece_begin(PieceState &st, const Dim &dm, float t0_ms, float traw, float v0x,
                                            float v0y, float v1x, float v1y) {
    const uint32_t tb = fbits(traw) & 0xFFFFFFFCu;
    st.t1_ms = (floorf(v1x) == v1x) ? ffrom(tb | 2u) : ffrom(tb | 3u);
    const CutRange cr = cut_range(v0x, v0y, v1x, v1y, dm.W, dm.H);
    st.nx = cr.nx;
    st.ny = cr.ny;
    st.n_loop = cr.nx + cr.ny + 1;
    st.x = (float)(cr.dx < 0.f ? cr.xe : cr.xb);
    st.y = (float)(cr.dy < 0.f ? cr.ye : cr.yb);
    st.dx = cr.dx;
    st.dy = cr.dy;
    st.slot0 = st.slot1 = t0_ms;
    st.last = fbits(-1.f);
    st.p = 0;
    st.i = -1;
}

// One step of a piece: the entry at the nearer of the two chains' current
// crossings (the piece start first), then the next crossing of that chain.
// Returns false once the piece is done.
__device__ __forceinline__ bool piece_step(PieceState &st) {
    float t_solve = 0.f, c = 0.f, t_min;
    int side = 0;
    if (st.i == -1) {
        t_min = st.slot0;
        if (st.nx == 0) {
            side = 0;
            t_solve = 2.f;
        } else if (st.ny == 0) {
            side = 1;
            t_solve = 2.f;
        } else {
            side = 0;
            st.nx--;
            c = st.x;
            st.x += st.dx;
        }
    } else if (st.slot0 <= st.slot1) {
        t_min = st.slot0;
        side = 0;
        if (st.nx > 0) {
            st.nx--;
            c = st.x;
            st.x += st.dx;
        } else {
            t_solve = 2.f;
        }
    } else {
        t_min = st.slot1;
        side = 1;
        if (st.ny > 0) {
            st.ny--;
            c = st.y;
            st.y += st.dy;
        } else {
            t_solve = 2.f;
        }
    }
    if (st.i >= 0) {
        uint32_t ob = fbits(t_min);
        if ((ob & 0xFFFFFFFCu) == (st.last & 0xFFFFFFFCu)) {  // coincident t: both entries get both flags
            ob |= st.last;
            st.out[st.p - 1] = make_int2(st.cid, (int)ob);
        }
        st.out[st.p] = make_int2(st.cid, (int)ob);
        st.last = ob;
        st.p++;
    }
    if (t_solve < 2.f) t_solve = solve_crossing(st.g, side ? st.g.py : st.g.px, c, t_min, st.t1_ms);
    const float sv = ffrom((fbits(t_solve) & 0xFFFFFFFCu) | (uint32_t)side);
    if (side) st.slot1 = sv;
    else st.slot0 = sv;
    return ++st.i < st.n_loop;
}

// Per warp: its 32 curves (in emission order), their monotone cut points
// and the output position of every piece.
constexpr int kEmitWarps = 4;
struct EmitStash {
    float px[4][32], py[4][32], w[32], q[5][32];
    uint32_t type[32], cid[32], poff[5][32];
    uint32_t item[5 * 32];  // warp item k: lane | piece << 8
};

// One warp per 32 curves.  Each lane expands its curve into its monotone
// pieces; the warp's pieces form one list, and a lane whose piece is done
// takes the next one (a ballot ranks the lanes asking), so the lanes stay
// busy until the list runs out instead of waiting for the curve with the
// most crossings.  Curves come in emission order (grouped by type), so a
// warp's pieces mostly run the same solver.
__global__ void __launch_bounds__(kEmitWarps * 32) k_curve_emit(FrameArgs a, const float2 *__restrict__ tv,
                                                                const uint8_t *__restrict__ vis,
                                                                const uint32_t *__restrict__ offsets,
                                                                const uint32_t *__restrict__ order,
                                                                int2 *__restrict__ entries,
                                                                const FrameCounters *__restrict__ ctr) {
    __shared__ EmitStash stash[kEmitWarps];
    // entries not admitted (the buffers are too small), or the offsets not
    // to be trusted (a scan gave up waiting): nothing is written
    if (ctr->status != 0u || ctr->nf != ctr->need_nf) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    EmitStash &S = stash[warp];
    const int i = (blockIdx.x * kEmitWarps + warp) * 32 + lane;
    int np = 0;
    if (i < a.C) {
        const int cid = order != nullptr ? (int)order[i] : i;
        const CurveDesc d = a.curves[cid];
        CurveGeom g;
        load_geom(d, tv, g);
        float q[5];
        np = monotonize_r(g, vis[d.pid] != 0, q);
        const Dim dm = dim_of(a, d.pid);
#pragma unroll
        for (int k = 0; k < 4; ++k) S.px[k][lane] = g.px[k], S.py[k][lane] = g.py[k];
        S.w[lane] = g.w;
        S.type[lane] = (uint32_t)g.type;
        S.cid[lane] = (uint32_t)cid;
        uint32_t run = offsets[cid];
        float v0x = g.px[0], v0y = g.py[0];
#pragma unroll
        for (int ms = 0; ms < 5; ++ms) {
            S.q[ms][lane] = q[ms];
            S.poff[ms][lane] = run;
            if (ms < np) {
                const float v1x = curve_coord(g.type, g.w, g.px, q[ms]), v1y = curve_coord(g.type, g.w, g.py, q[ms]);
                const CutRange cr = cut_range(v0x, v0y, v1x, v1y, dm.W, dm.H);
                run += 1 + cr.nx + cr.ny;
                v0x = v1x;
                v0y = v1y;
            }
        }
    }
    // the warp's piece list
    uint32_t pre = (uint32_t)np;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, pre, o);
        if (lane >= o) pre += v;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, pre, 31);
    pre -= (uint32_t)np;
    for (int ms = 0; ms < np; ++ms) S.item[pre + ms] = (uint32_t)lane | ((uint32_t)ms << 8);
    __syncwarp();
    PieceState st;
    bool active = false;
    uint32_t next = 0;
    for (;;) {
        const uint32_t want = __ballot_sync(0xffffffffu, !active);
        if (!active) {
            const uint32_t k = next + __popc(want & ((1u << lane) - 1u));
            if (k < total) {
                const uint32_t it = S.item[k];
                const int L = (int)(it & 0xFFu), ms = (int)(it >> 8);
                st.g.type = (int)S.type[L];
                st.g.w = S.w[L];
#pragma unroll
                for (int c = 0; c < 4; ++c) st.g.px[c] = S.px[c][L], st.g.py[c] = S.py[c][L];
                st.cid = (int)S.cid[L];
                st.out = entries + S.poff[ms][L];
                const float tq = S.q[ms][L];
                const float v1x = curve_coord(st.g.type, st.g.w, st.g.px, tq),
                            v1y = curve_coord(st.g.type, st.g.w, st.g.py, tq);
                float t0_ms = 0.f, v0x = st.g.px[0], v0y = st.g.py[0];
                if (ms > 0) {  // the previous piece's end: its parameter with its flags
                    const float tp = S.q[ms - 1][L];
                    v0x = curve_coord(st.g.type, st.g.w, st.g.px, tp);
                    v0y = curve_coord(st.g.type, st.g.w, st.g.py, tp);
                    const uint32_t tb = fbits(tp) & 0xFFFFFFFCu;
                    t0_ms = (floorf(v0x) == v0x) ? ffrom(tb | 2u) : ffrom(tb | 3u);
                }
                piece_begin(st, dim_of(a, a.curves[st.cid].pid), t0_ms, tq, v0x, v0y, v1x, v1y);
                active = true;
            }
        }
        next += __popc(want);
        if (!__any_sync(0xffffffffu, active)) break;
        if (active) active = piece_step(st);
    }
}

// ---------------------------------------------------------- fragments --
template <int S>
__global__ void __launch_bounds__(kThreads, 8) k_fragment(FrameArgs a, const float2 *__restrict__ tv,
                                                       const int2 *__restrict__ entries,
                                                       const FrameCounters *__restrict__ ctr,
                                                       int32_t *__restrict__ key_out, uint32_t *__restrict__ pid_out,
                                                       int8_t *__restrict__ wn_out, uint32_t *__restrict__ mask_out,
                                                       uint64_t *__restrict__ sort_key, uint32_t *__restrict__ sort_val) {
    constexpr int WORDS = S / 8;
    const int64_t nf = ctr->nf;
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
    const Dim dm = dim_of(a, pathid);
    int32_t yx = kInvalidKey;
    if (e0.x != e1.x) t1 = 1.f;
    int wnchg = 0, swn = 0;
    uint32_t mask[4] = {0u, 0u, 0u, 0u};
    float4 chord = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t lmk[4] = {0u, 0u, 0u, 0u};
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
        const int px = min(max(rx, -2), (int)(((uint32_t)dm.W & 0xFFFFFFFEu) + 2));
        const int py = min(max(ry, -2), (int)(((uint32_t)dm.H & 0xFFFFFFFEu) + 2));
        const uint32_t ys = (uint32_t)(py + 0x7FFF) << 16;
        const uint32_t xs = (uint32_t)(px + 0x7FFF) & 0xFFFFu;
        if ((uint32_t)ry < (uint32_t)dm.H) yx = (int32_t)(ys | xs);
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
        chord = make_float4(q0x, q0y, q1x, q1y);
#pragma unroll
        for (int w = 0; w < 4; ++w) lmk[w] = lm[w];
        uint32_t vm[4];
        vertical_mask2<S>(q0y, q1y, vm);
        const int texel = table_texel(q0x, q0y, q1x, q1y);
        if (S == 8) {
            const uint32_t tm = __ldg(a.mask_table + texel);
            mask[0] = (tm & vm[0]) ^ lm[0];
        } else if (S == 16) {
            const uint2 tm = __ldg(reinterpret_cast<const uint2 *>(a.mask_table) + texel);
            mask[0] = (tm.x & vm[0]) ^ lm[0];
            mask[1] = (tm.y & vm[1]) ^ lm[1];
        } else {
            const uint4 tm = __ldg(reinterpret_cast<const uint4 *>(a.mask_table) + texel);
            mask[0] = (tm.x & vm[0]) ^ lm[0];
            mask[1] = (tm.y & vm[1]) ^ lm[1];
            mask[2] = (tm.z & vm[2]) ^ lm[2];
            mask[3] = (tm.w & vm[3]) ^ lm[3];
        }
    }
    if (a.chord != nullptr) {
        a.chord[i] = chord;
        uint32_t vmk[4] = {0u, 0u, 0u, 0u};
        if (chord.y != chord.w) vertical_mask2<S>(chord.y, chord.w, vmk);
#pragma unroll
        for (int w = 0; w < WORDS; ++w) {
            a.lmask[i * WORDS + w] = lmk[w];
            a.vmask[i * WORDS + w] = vmk[w];
        }
    }
    key_out[i] = yx;
    pid_out[i] = pathid | ((uint32_t)wnchg << 30);
    wn_out[i] = (int8_t)swn;
    if (WORDS == 1) {
        mask_out[i] = mask[0];
    } else if (WORDS == 2) {
        reinterpret_cast<uint2 *>(mask_out)[i] = make_uint2(mask[0], mask[1]);
    } else {
        reinterpret_cast<uint4 *>(mask_out)[i] = make_uint4(mask[0], mask[1], mask[2], mask[3]);
    }
    const int nrows = (dm.H + 1) / 2;
    sort_key[i] = ((uint64_t)pathid << 24) | (uint64_t)local_sort_key(yx, nrows) |
                  ((uint64_t)pack_fw(swn, wnchg) << kFwShift);
    sort_val[i] = (uint32_t)i;
}

// --------------------------------------------- winding scan + marks --
constexpr int kMarkThreads = 256;
constexpr int kMarkItems = 8;
constexpr int kMarkTile = kMarkThreads * kMarkItems;
constexpr uint64_t kSegBit = 1ull << 32;  // winding look-back: a scene starts in the tile (batches)

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
    constexpr int W = kMarkThreads / 32;
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

// Segmented sums: (s, f) where f = a segment starts inside; a then b.
struct SegSum {
    uint32_t s, f;
};
__device__ __forceinline__ SegSum seg_then(SegSum a, SegSum b) { return SegSum{b.f ? b.s : a.s + b.s, a.f | b.f}; }

__device__ __forceinline__ SegSum block_excl_segscan(SegSum v, uint32_t *ss, uint32_t *sf, SegSum *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int W = kMarkThreads / 32;
    SegSum inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const SegSum up{__shfl_up_sync(0xffffffffu, inc.s, o), __shfl_up_sync(0xffffffffu, inc.f, o)};
        if (lane >= o) inc = seg_then(up, inc);
    }
    SegSum prev{__shfl_up_sync(0xffffffffu, inc.s, 1), __shfl_up_sync(0xffffffffu, inc.f, 1)};
    if (lane == 0) prev = SegSum{0u, 0u};
    if (lane == 31) ss[warp] = inc.s, sf[warp] = inc.f;
    __syncthreads();
    if (warp == 0) {
        SegSum t = lane < W ? SegSum{ss[lane], sf[lane]} : SegSum{0u, 0u};
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const SegSum up{__shfl_up_sync(0xffffffffu, t.s, o), __shfl_up_sync(0xffffffffu, t.f, o)};
            if (lane >= o) t = seg_then(up, t);
        }
        SegSum ex{__shfl_up_sync(0xffffffffu, t.s, 1), __shfl_up_sync(0xffffffffu, t.f, 1)};
        if (lane == 0) ex = SegSum{0u, 0u};
        if (lane < W) ss[lane] = ex.s, sf[lane] = ex.f;
        if (lane == W - 1) ss[W] = t.s, sf[W] = t.f;
    }
    __syncthreads();
    const SegSum r = seg_then(SegSum{ss[warp], sf[warp]}, prev);
    *total = SegSum{ss[W], sf[W]};
    __syncthreads();
    return r;
}

struct Mark {
    uint32_t ff, sf;
};

// Columns [x0, x1) of draw item `it` in a viewport W wide (its first column
// read as unsigned 16 bits: cells at x = -2 cover nothing).
__device__ __forceinline__ void item_cols(const int4 &it, int W, int &x0, int &x1) {
    const int x = (int)((uint32_t)it.x & 0xFFFFu);
    x0 = max(x, 0);
    x1 = min(x + it.y, W);
}

// Resolve bins of draw item `it` (the tiles of 1 << shift columns of the
// band of 64 >> shift cell rows holding its row) in a viewport W x H whose
// bins are numbered from bin0: *first and the count (consecutive bins).
__device__ __forceinline__ int item_bins(const int4 &it, int W, int H, int shift, uint32_t bin0, uint32_t *first) {
    int x0, x1;
    item_cols(it, W, x0, x1);
    const int row = (it.x >> 16) / 2;
    if (x1 <= x0 || row < 0 || row >= (H + 1) / 2) return 0;
    const int ntx = bin_cols(W, shift);
    *first = bin0 + (uint32_t)((row >> (kBinShift - shift)) * ntx + (x0 >> shift));
    return ((x1 - 1) >> shift) - (x0 >> shift) + 1;
}

// Counts item `it`'s pairs in its bins; returns its pairs in the other
// built-in tile (0 if there is none).
__device__ __forceinline__ uint32_t count_bins(const FrameArgs &a, const int4 &it, const Dim &dp, uint32_t p,
                                               uint32_t *__restrict__ bin_count) {
    const uint32_t bin0 = a.scenes != nullptr ? a.scenes[a.path_scene[p]].bin_off : 0u;
    uint32_t b0 = 0;
    const int nb = item_bins(it, dp.W, dp.H, a.bin_shift, bin0, &b0);
    for (int t = 0; t < nb; ++t) atomicAdd(bin_count + b0 + t, 1u);
    return a.alt_shift >= 0 ? (uint32_t)item_bins(it, dp.W, dp.H, a.alt_shift, 0u, &b0) : 0u;
}

// k_mark_merged_fragment_and_span (cu:462-535) on sorted position i with
// keys k0 (position i - 1) and k1 (position i) and scanned winding w.
__device__ __forceinline__ Mark mark_of(int64_t i, uint64_t k0, uint64_t k1, int8_t w, const FrameArgs &a) {
    const Dim dm = dim_of(a, (uint32_t)(k1 >> 24));
    const int W = dm.W, H = dm.H, nrows = (H + 1) / 2;
    const uint32_t key1 = (uint32_t)key_from_local((uint32_t)(k1 & 0xFFFFFFu), nrows);
    const int x1 = key_x(key1), y1 = key_y(key1);
    const bool oob = x1 < 0 || y1 < 0 || x1 >= W || y1 >= H;
    Mark m{0u, 0u};
    if (i == 0) {
        m.ff = oob ? 0u : 1u;
        return m;
    }
    const uint32_t p0 = (uint32_t)(k0 >> 24), p1 = (uint32_t)(k1 >> 24);
    const uint32_t key0 = (uint32_t)key_from_local((uint32_t)(k0 & 0xFFFFFFu), nrows);
    const int x0 = key_x(key0), y0 = key_y(key0);
    m.ff = oob ? 0u : ((p0 != p1 || key0 != key1) ? 1u : 0u);
    const uint8_t fr = a.fill_rule[p1];
    const bool wf = (fr == 0 && w != 0) || (fr == 1 && (w & 1));
    m.sf = (y0 == y1 && (x0 + 2) < x1 && p0 == p1 && wf) ? 1u : 0u;
    return m;
}

// Stages 9-12 and 14 in one pass over the sorted entries (thrust's int8
// scan of the shuffled windings, cu:1099-1101; the marks, cu:462-535; their
// inclusive scans, cu:1139-1157; the draw list, cu:789-868).  Per tile:
// the windings gathered through the sort permutation and scanned (int8
// arithmetic: only the low 8 bits are kept), with the tile's prefix from a
// decoupled look-back (restarting at every scene of a batch, so that each
// scene sees the scan a single-scene render gives it); then the merged and
// span marks, scanned with a second look-back, and the draw items written.
// The last tile writes the item counts.  Sorted keys are read 128 bits at a
// time; each carries its fragment's scan winding in bits 60-63.
__global__ void __launch_bounds__(kMarkThreads) k_scan_mark(FrameArgs a, const uint64_t *__restrict__ skey,
                                                            int8_t *__restrict__ wn_scan,
                                                            int4 *__restrict__ draw, uint32_t *__restrict__ heads,
                                                            uint32_t *__restrict__ item_scene,
                                                            uint32_t *__restrict__ bin_count,
                                                            FrameCounters *__restrict__ ctr,
                                                            uint64_t *__restrict__ st_wn, uint64_t *__restrict__ st_fl,
                                                            uint32_t spin_cap) {
    __shared__ uint32_t ss[kMarkThreads / 32 + 1], sf[kMarkThreads / 32 + 1];
    __shared__ uint32_t s_tile;
    __shared__ uint64_t s_pre;
    const int64_t nf = ctr->nf;
    const int64_t ntiles = (nf + kMarkTile - 1) / kMarkTile;
    if (threadIdx.x == 0) s_tile = atomicAdd(&ctr->tiles[1], 1u);
    __syncthreads();
    const int64_t t = s_tile;
    if (t >= ntiles) {
        if (t == 0 && threadIdx.x == 0) ctr->n_merged = ctr->n_span = ctr->n_items = 0u;
        return;
    }
    const int64_t base = t * kMarkTile + (int64_t)threadIdx.x * kMarkItems;
    const int64_t left = nf - base;
    const int cnt = left <= 0 ? 0 : (left >= kMarkItems ? kMarkItems : (int)left);
    uint64_t k[kMarkItems + 1];  // sorted keys at base - 1 .. base + 7
    if (cnt == kMarkItems) {
        const uint4 *kp = reinterpret_cast<const uint4 *>(skey + base);
#pragma unroll
        for (int q = 0; q < kMarkItems / 2; ++q) {
            const uint4 v = kp[q];
            k[1 + 2 * q] = (uint64_t)v.x | ((uint64_t)v.y << 32);
            k[2 + 2 * q] = (uint64_t)v.z | ((uint64_t)v.w << 32);
        }
    } else {
#pragma unroll
        for (int j = 0; j < kMarkItems; ++j) k[1 + j] = j < cnt ? skey[base + j] : 0ull;
    }
    k[0] = (cnt > 0 && base > 0) ? skey[base - 1] : 0ull;
    uint32_t fb[kMarkItems];  // the windings, and the keys without them
#pragma unroll
    for (int j = 0; j < kMarkItems; ++j) fb[j] = (uint32_t)(k[1 + j] >> kFwShift);
#pragma unroll
    for (int j = 0; j <= kMarkItems; ++j) k[j] &= kKeyMask;
    // windings in sorted order, and the scene starts of a batch
    const bool batch = a.scenes != nullptr && a.n_scenes > 1;
    int32_t v[kMarkItems];
    uint32_t seg = 0u;  // bit j: a scene starts at base + j
    SegSum agg{0u, 0u};
#pragma unroll
    for (int j = 0; j < kMarkItems; ++j) {
        v[j] = j < cnt ? fw_swn(fb[j]) : 0;
        if (batch && j < cnt &&
            (base + j == 0 || a.path_scene[(uint32_t)(k[j + 1] >> 24)] != a.path_scene[(uint32_t)(k[j] >> 24)]))
            seg |= 1u << j;
        agg = seg_then(agg, SegSum{(uint32_t)v[j], (seg >> j) & 1u});
    }
    SegSum tot;
    const SegSum tpre = block_excl_segscan(agg, ss, sf, &tot);
    if (threadIdx.x < 32) {
        uint64_t pre = 0;
        if (t > 0) {
            if (threadIdx.x == 0) lb_store(st_wn + t, kLbAggregate | (tot.f ? kSegBit : 0ull) | tot.s);
            pre = lb_walk(st_wn, t, kSegBit, spin_cap, &ctr->status);
        }
        if (threadIdx.x == 0) {
            lb_store(st_wn + t, kLbInclusive | (uint32_t)(tot.f ? tot.s : (uint32_t)pre + tot.s));
            s_pre = pre;
        }
    }
    __syncthreads();
    // scanned windings (exclusive, restarting at scene starts)
    SegSum run = seg_then(SegSum{(uint32_t)s_pre, 0u}, tpre);
    int8_t ws[kMarkItems];
#pragma unroll
    for (int j = 0; j < kMarkItems; ++j) {
        if ((seg >> j) & 1u) run.s = 0u;
        ws[j] = (int8_t)(uint8_t)run.s;
        run.s += (uint32_t)v[j];
    }
    if (cnt == kMarkItems) {
        uint2 packed;
        packed.x = (uint32_t)(uint8_t)ws[0] | ((uint32_t)(uint8_t)ws[1] << 8) | ((uint32_t)(uint8_t)ws[2] << 16) |
                   ((uint32_t)(uint8_t)ws[3] << 24);
        packed.y = (uint32_t)(uint8_t)ws[4] | ((uint32_t)(uint8_t)ws[5] << 8) | ((uint32_t)(uint8_t)ws[6] << 16) |
                   ((uint32_t)(uint8_t)ws[7] << 24);
        *reinterpret_cast<uint2 *>(wn_scan + base) = packed;
    } else {
#pragma unroll
        for (int j = 0; j < kMarkItems; ++j)
            if (j < cnt) wn_scan[base + j] = ws[j];
    }
    // marks and their scans
    Mark mk[kMarkItems];
    uint32_t fs = 0;
#pragma unroll
    for (int j = 0; j < kMarkItems; ++j) {
        mk[j] = j < cnt ? mark_of(base + j, k[j], k[j + 1], ws[j], a) : Mark{0u, 0u};
        fs += mk[j].ff | (mk[j].sf << 16);
    }
    uint32_t ftot;
    const uint32_t fpre = block_excl_scan(fs, ss, &ftot);
    const uint64_t ftot_w = ((uint64_t)(ftot & 0xFFFFu) << 31) | (uint64_t)(ftot >> 16);
    if (threadIdx.x < 32) {
        uint64_t pre = 0;
        if (t > 0) {
            if (threadIdx.x == 0) lb_store(st_fl + t, kLbAggregate | ftot_w);
            pre = lb_walk(st_fl, t, 0ull, spin_cap, &ctr->status);
        }
        if (threadIdx.x == 0) {
            lb_store(st_fl + t, kLbInclusive | ((pre + ftot_w) & kLbPayload));
            s_pre = pre;
            if (t == ntiles - 1) {  // the frame's item counts
                const uint64_t all = pre + ftot_w;
                const uint32_t nm = (uint32_t)(all >> 31) & 0x7FFFFFFFu, ns = (uint32_t)all & 0x7FFFFFFFu;
                ctr->n_merged = nm;
                ctr->n_span = ns;
                ctr->n_items = nm + ns;
            }
        }
    }
    __syncthreads();
    uint32_t nfb = (uint32_t)(s_pre >> 31) + (fpre & 0xFFFFu);
    uint32_t nsb = (uint32_t)(s_pre & 0x7FFFFFFFu) + (fpre >> 16);
    uint32_t span_px = 0, pairs_alt = 0;  // this thread's span pixels and pairs in the other tile
#pragma unroll
    for (int j = 0; j < kMarkItems; ++j) {
        const uint32_t ff = mk[j].ff, sfl = mk[j].sf;
        if (ff | sfl) {
            const uint64_t k1 = k[j + 1];
            const uint32_t p = (uint32_t)(k1 >> 24);
            const int32_t fill = (int32_t)a.fill_rgba[p];
            const Dim dp = dim_of(a, p);
            const int nrows = (dp.H + 1) / 2;
            const uint32_t key1 = (uint32_t)key_from_local((uint32_t)(k1 & 0xFFFFFFu), nrows);
            if (item_scene != nullptr) {
                const uint32_t sc = a.path_scene[p];
                if (ff) item_scene[nfb + nsb] = sc;
                if (sfl) item_scene[nfb + nsb + ff] = sc;
            }
            if (a.item_path != nullptr) {
                if (ff) a.item_path[nfb + nsb] = p;
                if (sfl) a.item_path[nfb + nsb + ff] = p;
            }
            if (ff) {
                const int32_t pos = (int32_t)(((uint32_t)key_y(key1) << 16) | (uint32_t)key_x(key1));
                const int4 it = make_int4(pos, 2, fill, (int)(nfb + 1));
                draw[nfb + nsb] = it;
                pairs_alt += count_bins(a, it, dp, p, bin_count);
                heads[nfb] = (uint32_t)(base + j);
            }
            if (sfl) {
                const uint32_t key0 = (uint32_t)key_from_local((uint32_t)(k[j] & 0xFFFFFFu), nrows);
                const int y0 = key_y(key0);
                int x0 = (int16_t)(key_x(key0) + 2);
                const int x1 = key_x(key1);
                x0 = max(0, x0);
                const int32_t pos = (int32_t)(((uint32_t)y0 << 16) | (uint32_t)x0);
                const int4 it = make_int4(pos, x1 - x0, fill, 0);
                draw[nfb + nsb + ff] = it;
                pairs_alt += count_bins(a, it, dp, p, bin_count);
                span_px += (uint32_t)max(x1 - x0, 0);
            }
        }
        nfb += ff;
        nsb += sfl;
    }
    const uint32_t wpx = __reduce_add_sync(0xffffffffu, span_px);
    const uint32_t wpa = __reduce_add_sync(0xffffffffu, pairs_alt);
    if ((threadIdx.x & 31) == 0 && wpx) atomicAdd(&ctr->span_px, (unsigned long long)wpx);
    if ((threadIdx.x & 31) == 0 && wpa) atomicAdd(&ctr->pairs_alt, wpa);
}

// ------------------------------------------------------- merged masks --
// Per merged fragment: the scanned winding number plus the signed boundary
// masks of every fragment of the (path, cell) group, in 8-bit lanes per
// mask bit (the reference's packed counters), reduced to the 7-bit winding
// number and tested against the fill rule.
//
// A block takes 256 consecutive merged fragments, whose groups are one
// contiguous run of sorted positions [heads[g0], heads[g0 + 256]).  The run
// (up to kStencilStage positions, from a 16-entry boundary) is staged into
// shared memory by bulk copies (cp.async.bulk, completion on an mbarrier)
// of the sorted keys (with the change signs in bits 60-63) and fragment
// indices; positions past the staged run are read from global memory.  The
// sample masks are read through the fragment indices.
constexpr int kStencilStage = 1024;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// Waits for phase 0 of mbarrier `bar`, at most `cap` polls; false if it
// did not complete.
__device__ __forceinline__ bool mbar_wait0(uint32_t bar, uint32_t cap) {
    for (uint32_t it = 0; it < cap; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, "
            "p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(0u)
            : "memory");
        if (done) return true;
    }
    return false;
}

struct StencilStage {
    uint64_t key[kStencilStage];
    uint32_t perm[kStencilStage];
    uint64_t bar;
};

template <int S>
__global__ void __launch_bounds__(kThreads, 5) k_stencil(FrameArgs a, FrameCounters *__restrict__ ctr,
                                                      const uint64_t *__restrict__ skey,
                                                      const uint32_t *__restrict__ perm,
                                                      const uint32_t *__restrict__ mask,
                                                      const int8_t *__restrict__ wn_scan,
                                                      const uint32_t *__restrict__ heads,
                                                      uint32_t *__restrict__ merged, uint32_t spin_cap) {
    constexpr int WORDS = S / 8;
    __shared__ __align__(16) StencilStage st;
    const int64_t nf = ctr->nf, nm = ctr->n_merged;
    const int64_t g0 = (int64_t)blockIdx.x * blockDim.x;
    if (g0 >= nm) return;
    // the block's run of sorted positions, from a 16-entry boundary
    const int64_t s16 = (int64_t)heads[g0] & ~(int64_t)15;
    const int64_t e = g0 + (int64_t)blockDim.x < nm ? (int64_t)heads[g0 + blockDim.x] : nf;
    const int64_t e16 = (e + 15) & ~(int64_t)15;
    const int64_t n_st = min(e16 - s16, (int64_t)kStencilStage);  // a multiple of 16
    const uint32_t bar = smem_addr(&st.bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = (uint32_t)n_st * (8u + 4u);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
        bulk_g2s(st.key, skey + s16, (uint32_t)n_st * 8u, bar);
        bulk_g2s(st.perm, perm + s16, (uint32_t)n_st * 4u, bar);
    }
    // this thread's group head and its scanned winding, while the copies run
    const int64_t g = g0 + threadIdx.x;
    const bool live = g < nm;
    const int64_t h = live ? (int64_t)heads[g] : 0;
    const int32_t w0 = live ? (int32_t)wn_scan[h] : 0;
    if (!mbar_wait0(bar, spin_cap)) {
        if (threadIdx.x == 0) atomicOr(&ctr->status, kStatusTimeout);
        mbar_wait0(bar, spin_cap);  // the copies still in flight write this block's shared memory
        return;
    }
    if (!live) return;
    auto key_at = [&](int64_t j) { return j - s16 < n_st ? st.key[j - s16] : skey[j]; };
    const uint64_t kh = key_at(h) & kKeyMask;
    // the group's fragments with a winding change: fn(change sign, mask)
    auto walk = [&](auto &&fn) {
        for (int64_t j = h; j < nf; ++j) {
            const bool staged = j - s16 < n_st;
            const uint64_t kj = staged ? st.key[j - s16] : skey[j];
            if ((kj & kKeyMask) != kh) break;
            const int32_t chg = fw_chg((uint32_t)(kj >> kFwShift));
            if (chg == 0) continue;
            const uint32_t raw = staged ? st.perm[j - s16] : perm[j];
            uint32_t m[WORDS];
            if constexpr (WORDS == 1) {
                m[0] = __ldg(mask + raw);
            } else if constexpr (WORDS == 2) {
                const uint2 v = __ldg(reinterpret_cast<const uint2 *>(mask) + raw);
                m[0] = v.x;
                m[1] = v.y;
            } else {
                const uint4 v = __ldg(reinterpret_cast<const uint4 *>(mask) + raw);
                m[0] = v.x;
                m[1] = v.y;
                m[2] = v.z;
                m[3] = v.w;
            }
            fn(chg, m);
        }
    };
    const int fr = a.fill_rule[(uint32_t)(kh >> 24)];
    // Every sample's winding w0 + (sum of the changes of the fragments covering
    // it) as a 7-bit counter, bit-sliced: plane p holds bit p of the counters of
    // all samples, and adding a fragment is a ripple carry (or borrow) over the
    // planes.  The packed counters below (four 8-bit counters per word, the
    // reference's form) give each sample its winding modulo 128 as long as no
    // winding leaves [-128, 127], where a byte's carry would reach its
    // neighbour; with |w0| + (fragments) <= 127 that cannot happen, and the
    // planes give the same bits.
    uint32_t pl[7][WORDS];
#pragma unroll
    for (int q = 0; q < 7; ++q)
#pragma unroll
        for (int w = 0; w < WORDS; ++w) pl[q][w] = (((uint32_t)w0 >> q) & 1u) ? 0xFFFFFFFFu : 0u;
    int k = 0;
    walk([&](int32_t chg, const uint32_t (&m)[WORDS]) {
        ++k;
#pragma unroll
        for (int w = 0; w < WORDS; ++w) {
            uint32_t c = m[w];
            if (chg > 0) {
#pragma unroll
                for (int q = 0; q < 7; ++q) {
                    const uint32_t t = pl[q][w] & c;
                    pl[q][w] ^= c;
                    c = t;
                }
            } else {
#pragma unroll
                for (int q = 0; q < 7; ++q) {
                    const uint32_t t = ~pl[q][w] & c;
                    pl[q][w] ^= c;
                    c = t;
                }
            }
        }
    });
    if ((w0 < 0 ? -w0 : w0) + k <= 127) {
#pragma unroll
        for (int w = 0; w < WORDS; ++w) {
            // nonzero: any bit of the 7-bit winding; even-odd: its lowest bit
            const uint32_t ret = fr == 0 ? (pl[0][w] | pl[1][w] | pl[2][w] | pl[3][w] | pl[4][w] | pl[5][w] | pl[6][w])
                                         : pl[0][w];
            merged[g * WORDS + w] = ret;
        }
        return;
    }
    // packed 8-bit counters per mask bit, reduced to the 7-bit winding number
    const uint32_t init = 0x01010101u * (uint32_t)w0;
    uint32_t acc[WORDS][8];
#pragma unroll
    for (int w = 0; w < WORDS; ++w)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[w][b] = init;
    walk([&](int32_t chg, const uint32_t (&m)[WORDS]) {
#pragma unroll
        for (int w = 0; w < WORDS; ++w)
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                const uint32_t bits = (m[w] >> b) & 0x01010101u;
                acc[w][b] = chg > 0 ? acc[w][b] + bits : acc[w][b] - bits;
            }
    });
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
constexpr int kResolveWarps = 8;
constexpr int kResolveMaxBlocksPerSM = 4;

// The draw items of every resolve bin, in draw order: each item's index is
// placed in its bins' ranges (bin offsets from the scan of the counts that
// k_scan_mark took) by warp-aggregated atomic slots, and every bin's range
// is then sorted (item indices are the draw order).
__global__ void k_bin_scatter(FrameArgs a, const int4 *__restrict__ draw, const uint32_t *__restrict__ item_scene,
                              const FrameCounters *__restrict__ ctr, const uint32_t *__restrict__ bin_off,
                              uint32_t *__restrict__ bin_fill, uint32_t *__restrict__ pval) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    // (pairs not admitted: the pair buffer is too small; or a scan gave up)
    const bool ok = ctr->status == 0u && ctr->n_pairs == ctr->need_pairs;
    int nb = 0;
    uint32_t b0 = 0;
    if (ok && i < (int64_t)ctr->n_items) {
        const int4 it = draw[i];
        int W = a.W, H = a.H;
        uint32_t bin0 = 0;
        if (item_scene != nullptr) {
            const SceneInfo *sc = a.scenes + item_scene[i];
            W = sc->W;
            H = sc->H;
            bin0 = sc->bin_off;
        }
        nb = item_bins(it, W, H, a.bin_shift, bin0, &b0);
    }
    const int most = __reduce_max_sync(0xffffffffu, nb);
    for (int t = 0; t < most; ++t) {
        const bool act = t < nb;
        const uint32_t bin = act ? b0 + (uint32_t)t : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xffffffffu, bin);
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (act && lane == leader) base = atomicAdd(bin_fill + bin, (uint32_t)__popc(peers));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (act) pval[bin_off[bin] + base + __popc(peers & ((1u << lane) - 1u))] = (uint32_t)i;
    }
}

// Pairs of every bin counted again from the draw list (a sized frame that
// changes its resolve tile after the scan-mark pass counted them).
__global__ void k_bin_count(FrameArgs a, const int4 *__restrict__ draw, const uint32_t *__restrict__ item_scene,
                            const FrameCounters *__restrict__ ctr, uint32_t *__restrict__ bin_count) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ctr->status != 0u || i >= (int64_t)ctr->n_items) return;
    const int4 it = draw[i];
    int W = a.W, H = a.H;
    uint32_t bin0 = 0;
    if (item_scene != nullptr) {
        const SceneInfo *sc = a.scenes + item_scene[i];
        W = sc->W;
        H = sc->H;
        bin0 = sc->bin_off;
    }
    uint32_t b0 = 0;
    const int nb = item_bins(it, W, H, a.bin_shift, bin0, &b0);
    for (int t = 0; t < nb; ++t) atomicAdd(bin_count + b0 + t, 1u);
}

// One warp per bin: its item indices sorted ascending by a bitonic network
// that compares in one direction only (stage k compares each element with
// its mirror in the k-block, then the half-cleaners), so that the missing
// elements past n behave as +infinity.  Bins of up to kBinSortSmem items are
// sorted in shared memory, larger ones in place.  With rec_a set, the bin's
// resolve records are written in the same order: the item's colour, its
// columns and cell row within the bin's band (first | width << 16 |
// row << 29) and its merged sample mask (every sample for a span), so that
// the resolve reads each bin's items and masks as one contiguous run
// instead of gathering them.  (Widths stay below 2^13: viewports are at
// most 4096 pixels wide.)
constexpr int kBinSortWarps = 4;
constexpr int kBinSortSmem = 1024;
template <int MW>
struct MaskVec;
template <>
struct MaskVec<1> {
    using T = uint32_t;
    static __device__ __forceinline__ T all() { return 0xFFFFFFFFu; }
};
template <>
struct MaskVec<2> {
    using T = uint2;
    static __device__ __forceinline__ T all() { return make_uint2(0xFFFFFFFFu, 0xFFFFFFFFu); }
};
template <>
struct MaskVec<4> {
    using T = uint4;
    static __device__ __forceinline__ T all() { return make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu); }
};

template <int MW>
__global__ void __launch_bounds__(kBinSortWarps * 32)
    k_bin_sort(const uint32_t *__restrict__ bin_off, int64_t nbins, uint32_t *__restrict__ pval,
               const FrameCounters *__restrict__ ctr, const int4 *__restrict__ draw,
               const uint32_t *__restrict__ merged, uint2 *__restrict__ rec_a,
               typename MaskVec<MW>::T *__restrict__ rec_m, int band_mask) {
    using MV = typename MaskVec<MW>::T;
    __shared__ uint32_t sk[kBinSortWarps][kBinSortSmem];
    if (ctr->status != 0u || ctr->n_pairs != ctr->need_pairs) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t b = (int64_t)blockIdx.x * kBinSortWarps + warp;
    if (b >= nbins) return;
    const uint32_t beg = bin_off[b], n = bin_off[b + 1] - beg;
    if (n == 0u) return;
    const bool in_smem = n <= (uint32_t)kBinSortSmem;
    uint32_t *k = in_smem ? sk[warp] : pval + beg;
    if (n > 1u) {
        if (in_smem) {
            for (uint32_t i = lane; i < n; i += 32) k[i] = pval[beg + i];
            __syncwarp();
        }
        int lp = 1;
        while ((1u << lp) < n) ++lp;  // 2^lp >= n
        const uint32_t half = 1u << (lp - 1);
        for (int lk = 1; lk <= lp; ++lk) {
            for (int lj = lk - 1; lj >= 0; --lj) {
                const uint32_t j = 1u << lj;
                for (uint32_t i = lane; i < half; i += 32) {
                    uint32_t x, y;
                    if (lj == lk - 1) {  // mirror within the 2j-block
                        const uint32_t blk = (i >> lj) << lk, off = i & (j - 1u);
                        x = blk + off;
                        y = blk + (2u * j - 1u) - off;
                    } else {
                        x = ((i >> lj) << (lj + 1)) + (i & (j - 1u));
                        y = x + j;
                    }
                    if (y < n) {
                        const uint32_t u = k[x], v = k[y];
                        if (u > v) {
                            k[x] = v;
                            k[y] = u;
                        }
                    }
                }
                __syncwarp();
            }
        }
        if (in_smem)
            for (uint32_t i = lane; i < n; i += 32) pval[beg + i] = k[i];
    }
    if (rec_a == nullptr) return;
    for (uint32_t i = lane; i < n; i += 32) {
        const uint32_t idx = n > 1u ? k[i] : pval[beg];
        const int4 it = draw[idx];
        const uint32_t ro = (uint32_t)(((it.x >> 16) / 2) & band_mask);  // the item's cell row within the band
        rec_a[beg + i] = make_uint2((uint32_t)it.z,
                                    ((uint32_t)it.x & 0xFFFFu) | ((uint32_t)it.y << 16) | (ro << 29));
        rec_m[beg + i] = it.w != 0 ? reinterpret_cast<const MV *>(merged)[it.w - 1] : MaskVec<MW>::all();
    }
}

// Shared-memory tables of the resolve.  The sRGB decode table is replicated
// twice (entry k of lane l at k * 2 + l % 2), which measures as fast as more
// replicas and leaves the room for 4 resolve blocks per SM.
struct SmemTables {
    float dec8r[256 * 2];
    float th[256];
    uint8_t bin[4096];  // number of thresholds <= b / 4096
};

__device__ __forceinline__ float lin8(uint32_t k) { return (float)k * (1.f / 255.f); }

// Blend results are finite and never -0 (products and sums of non-negative
// values), so the hardware min/max give the same clamp as fmin_r/fmax_r.
__device__ __forceinline__ float clamp01(float v) { return fminf(fmaxf(v, 0.f), 1.f); }

__device__ __forceinline__ uint32_t enc_lin(float v) {
    const float c = clamp01(v);
    return (uint32_t)cvt_rzi(c * 255.f + 0.5f);
}

// sRGB encode: the number of thresholds t[k] (the linear value at which the
// 8-bit code steps from k to k+1) that are <= v.  The thresholds are at
// least 3.0e-4 apart, wider than the 1/4096 bins of `bin`, so a bin holds at
// most one of them: the count is the bin's base plus one comparison.
__device__ __forceinline__ uint32_t enc_srgb(const SmemTables &t, float v) {
    const float c = clamp01(v);
    const int b = min(cvt_rzi(c * 4096.f), 4095);
    uint32_t k = t.bin[b];
    if (k < 255u && c >= t.th[k]) ++k;
    return k;
}

template <bool SRGB>
__device__ __forceinline__ float dec8(const SmemTables &t, uint32_t k, int lane) {
    if constexpr (SRGB) return t.dec8r[k * 2 + (lane & 1)];
    else return lin8(k);
}

template <bool SRGB>
__device__ __forceinline__ uint32_t enc8(const SmemTables &t, float v) {
    if constexpr (SRGB) return enc_srgb(t, v);
    else return enc_lin(v);
}

template <bool SRGB>
__device__ __forceinline__ uint32_t blend_sample(const SmemTables &t, int lane, uint32_t dv, float sr, float sg,
                                                 float sb, float a, float om) {
    const float dr = dec8<SRGB>(t, dv & 0xFF, lane), dg = dec8<SRGB>(t, (dv >> 8) & 0xFF, lane),
                db = dec8<SRGB>(t, (dv >> 16) & 0xFF, lane);
    const float da = lin8(dv >> 24);
    const float orr = sr * a + dr * om;
    const float og = sg * a + dg * om;
    const float ob = sb * a + db * om;
    const float oa = a * a + da * om;
    return enc8<SRGB>(t, orr) | (enc8<SRGB>(t, og) << 8) | (enc8<SRGB>(t, ob) << 16) | (enc_lin(oa) << 24);
}

// ---- gradient paints -----------------------------------------------------
// Gradient coordinate of pixel position (x, y): back to the scene through
// the reverse transform, then the entry's 2x3 map (ms_output_32.vert.glsl
// calc_color).
__device__ __forceinline__ float2 grad_coord(const FrameArgs &a, const float4 &w0, const float4 &w1, float x, float y) {
    const float rdx = (a.rev[0] * x + a.rev[3] * y) + a.rev[6];
    const float rdy = (a.rev[1] * x + a.rev[4] * y) + a.rev[7];
    const float rdz = (a.rev[2] * x + a.rev[5] * y) + a.rev[8];
    const float k = a.rev[12] / rdz;
    const float ox = a.rev[9] + k * rdx, oy = a.rev[10] + k * rdy;
    return make_float2((ox * w0.x + oy * w0.y) + w0.z, (ox * w0.w + oy * w1.x) + w1.y);
}

// Colour of gradient entry e at the centre of pixel (X, Y) for a draw item
// starting at column x0, w pixels wide: the coordinate interpolated along
// the item's row between its ends (the GL line primitive), the focal-point
// ratio c, and the ramp sampled at c (n - 1) texels past the first with
// linear filtering (ms_output_32.frag.glsl).  Texels are decoded from sRGB
// first under sRGB blending.
template <bool SRGB>
__device__ __forceinline__ float4 gradient_colour(const FrameArgs &a, const SmemTables &T, uint32_t e, int x0, int w,
                                                  int X, int Y, int lane) {
    const float4 w0 = a.grad_table[3 * e], w1 = a.grad_table[3 * e + 1], w2 = a.grad_table[3 * e + 2];
    const float yr = (float)Y + 0.5f;
    const float2 g0 = grad_coord(a, w0, w1, (float)x0, yr), g1 = grad_coord(a, w0, w1, (float)(x0 + w), yr);
    const float t = ((float)X + 0.5f - (float)x0) / (float)w;
    const float gx = g0.x * (1.f - t) + g1.x * t, gy = g0.y * (1.f - t) + g1.y * t;
    const float dx = gx - w2.x, dy = gy - w2.y;
    const float A = dx * dx + dy * dy, B = dx * w2.x + dy * w2.y;
    const float den = sqrtf(B * B + A * w2.z) - B;
    const float c = fminf(A * (den > 1e-6f ? 1.f / den : 0.f), 1.f);
    const int p = __float_as_int(w1.z);
    const float pos = c * (w1.w * 1024.f);
    const int i0 = (int)floorf(pos);
    const float f = pos - (float)i0;
    const int row = p >> 10, col = min((p & 1023) + i0, 1023), col1 = min(col + 1, 1023);
    const uint32_t t0 = a.grad_ramp[row * 1024 + col], t1 = a.grad_ramp[row * 1024 + col1];
    const float u = 1.f - f;
    return make_float4(dec8<SRGB>(T, t0 & 0xFF, lane) * u + dec8<SRGB>(T, t1 & 0xFF, lane) * f,
                       dec8<SRGB>(T, (t0 >> 8) & 0xFF, lane) * u + dec8<SRGB>(T, (t1 >> 8) & 0xFF, lane) * f,
                       dec8<SRGB>(T, (t0 >> 16) & 0xFF, lane) * u + dec8<SRGB>(T, (t1 >> 16) & 0xFF, lane) * f,
                       lin8(t0 >> 24) * u + lin8(t1 >> 24) * f);
}

// ---- resolve state -------------------------------------------------------
// A bin is one cell row (2 pixel rows) x 64 pixel columns = 32 cells of 2x2
// pixels; lane l of the warp resolving the bin owns cell l.  Every draw item
// covers whole cells, and the 4 pixels of a cell see the same items in the
// same order, so a cell keeps its 4 x S samples (pixel k = px.x * 2 + px.y,
// the merged masks' layout: bits [k S, (k + 1) S) of the cell's mask words)
// as a short list of (sample mask, RGBA8 colour) entries whose masks
// partition the samples.  An item blends each entry it touches once,
// splitting the entries it covers in part, and entries of equal colour are
// merged after every item: a cell typically holds 1-4 entries, and an entry
// often spans several pixels, so one blend serves many samples.  Entries
// 0..kCellCap-1 live in shared memory; a cell that needs more (rare: up to
// one per sample) keeps the rest in a global area owned by its warp and
// lane, with the same layout.  Every sample gets exactly the value the
// per-sample rule gives.
constexpr int kCellCap = 8;

// Draw items per window: kWin batches of 32.
constexpr int kWin = 8;

template <int MW, int CAP>
struct CellState {
    uint32_t ent[CAP][MW + 1][32];  // entry j of lane l's cell: mask words k < MW, colour at k = MW
    uint32_t mine[kWin][32];        // per batch, the window's items covering lane l's cell
};

// Entry j of lane `lane`'s cell: its first word; word k is at [k * 32].
template <int MW, int CAP>
__device__ __forceinline__ uint32_t *entry(CellState<MW, CAP> &w, uint32_t *gx, int j, int lane) {
    return j < CAP ? &w.ent[j][0][lane] : gx + (size_t)(j - CAP) * (MW + 1) * 32 + lane;
}

// Cells [c0, c1) of cell row `ro` of a bin whose rows hold cpr cells (lane
// ro * cpr + c holds cell c of row ro) as a lane mask.
__device__ __forceinline__ uint32_t cell_bits(int c0, int c1, int cpr, int ro) {
    c0 = max(c0, 0);
    c1 = min(c1, cpr);
    if (c1 <= c0) return 0u;
    const uint32_t hi = c1 >= 32 ? 0xFFFFFFFFu : ((1u << c1) - 1u);
    return (hi & ~((1u << c0) - 1u)) << (ro * cpr);
}

// Bits of pixel k within mask word `wd` (cell masks of S samples per pixel).
template <int S>
__device__ __forceinline__ uint32_t pixel_word_bits(int wd, int k) {
    if constexpr (S == 32) return wd == k ? 0xFFFFFFFFu : 0u;
    else if constexpr (S == 16) return wd == (k >> 1) ? (0xFFFFu << (16 * (k & 1))) : 0u;
    else return 0xFFu << (8 * k);
}

// Merges entries of equal colour.
template <int MW, int CAP>
__device__ __forceinline__ void cell_dedup(CellState<MW, CAP> &w, uint32_t *gx, int lane, int &n) {
    for (int j = 1; j < n; ++j) {
        uint32_t *ej = entry(w, gx, j, lane);
        const uint32_t cj = ej[MW * 32];
        for (int i = 0; i < j; ++i) {
            uint32_t *ei = entry(w, gx, i, lane);
            if (ei[MW * 32] == cj) {
                --n;
                uint32_t *en = entry(w, gx, n, lane);
#pragma unroll
                for (int k = 0; k < MW; ++k) {
                    ei[k * 32] |= ej[k * 32];
                    ej[k * 32] = en[k * 32];
                }
                ej[MW * 32] = en[MW * 32];
                --j;
                break;
            }
        }
    }
}

// One item (source colour sr, sg, sb with alpha sa) over the samples of mask
// m of lane `lane`'s cell, in the multisample modes.
template <int S, bool SRGB, int CAP>
__device__ __forceinline__ void cell_apply(CellState<S / 8, CAP> &w, uint32_t *gx, int lane, int &n,
                                           const uint32_t (&m)[S / 8], const SmemTables &T, float sr, float sg,
                                           float sb, float sa) {
    constexpr int MW = S / 8;
    const float om = 1.f - sa;
    uint32_t full = 0xFFFFFFFFu;
#pragma unroll
    for (int k = 0; k < MW; ++k) full &= m[k];
    if (sa == 1.f && full == 0xFFFFFFFFu) {
        // opaque over every sample: src * 1 + dst * 0 is the source whatever
        // dst holds, so one entry stands for all (the per-sample blends and
        // the merge give the same)
        uint32_t *e0 = &w.ent[0][0][lane];
        e0[MW * 32] = blend_sample<SRGB>(T, lane, 0u, sr, sg, sb, sa, om);
#pragma unroll
        for (int k = 0; k < MW; ++k) e0[k * 32] = 0xFFFFFFFFu;
        n = 1;
        return;
    }
    const int n0 = n;
    bool changed = false;
    for (int j = 0; j < n0; ++j) {
        uint32_t *ej = entry(w, gx, j, lane);
        uint32_t em[MW], in[MW], any = 0u, part = 0u;
#pragma unroll
        for (int k = 0; k < MW; ++k) {
            em[k] = ej[k * 32];
            in[k] = em[k] & m[k];
            any |= in[k];
            part |= em[k] & ~m[k];
        }
        if (!any) continue;
        const uint32_t r = blend_sample<SRGB>(T, lane, ej[MW * 32], sr, sg, sb, sa, om);
        changed = true;
        if (!part) {
            ej[MW * 32] = r;
        } else {
            uint32_t *en = entry(w, gx, n, lane);
#pragma unroll
            for (int k = 0; k < MW; ++k) {
                ej[k * 32] = em[k] & ~m[k];
                en[k * 32] = in[k];
            }
            en[MW * 32] = r;
            ++n;
        }
    }
    if (changed && n > 1) cell_dedup<MW, CAP>(w, gx, lane, n);
}

// Sample mask m (MW words) of resolve record p.
template <int MW>
__device__ __forceinline__ void load_mask(const uint32_t *__restrict__ rec_m, uint32_t p, uint32_t (&m)[MW]) {
    if constexpr (MW == 4) {
        const uint4 v = __ldg(reinterpret_cast<const uint4 *>(rec_m) + p);
        m[0] = v.x, m[1] = v.y, m[2] = v.z, m[3] = v.w;
    } else if constexpr (MW == 2) {
        const uint2 v = __ldg(reinterpret_cast<const uint2 *>(rec_m) + p);
        m[0] = v.x, m[1] = v.y;
    } else {
        m[0] = __ldg(rec_m + p);
    }
}

// Exact mean of a pixel's samples: every decoded value x 2^36 is an integer,
// the 64-bit sums are exact, one rounding to float at the end.
struct PixelSum {
    long long r = 0, g = 0, b = 0, a = 0;
};
template <bool SRGB>
__device__ __forceinline__ void add_sample(PixelSum &p, const SmemTables &T, int lane, uint32_t v, int weight) {
    p.r += (long long)weight * (long long)(dec8<SRGB>(T, v & 0xFF, lane) * 68719476736.0f);
    p.g += (long long)weight * (long long)(dec8<SRGB>(T, (v >> 8) & 0xFF, lane) * 68719476736.0f);
    p.b += (long long)weight * (long long)(dec8<SRGB>(T, (v >> 16) & 0xFF, lane) * 68719476736.0f);
    p.a += (long long)weight * (long long)(lin8(v >> 24) * 68719476736.0f);
}

template <bool SRGB>
__device__ __forceinline__ uint32_t encode_mean(const SmemTables &T, const PixelSum &p, double scale) {
    const float ar = (float)((double)p.r * scale), ag = (float)((double)p.g * scale);
    const float ab = (float)((double)p.b * scale), aa = (float)((double)p.a * scale);
    return enc8<SRGB>(T, ar) | (enc8<SRGB>(T, ag) << 8) | (enc8<SRGB>(T, ab) << 16) | (enc_lin(aa) << 24);
}

// One warp per bin.  The bin's resolve records (merged fragments and spans
// in draw-list order: colour, columns, sample mask) are taken kWin x 32 at a
// time; a 32 x 32 ballot transpose of each batch's cell sets gives every
// lane the window's items covering its cell, which it applies in order,
// independently of the other lanes until the window ends (a lane's work is
// the items over its own cell, not the most any lane has in each batch).
// The record of the lane's next item is loaded while it applies the current
// one.  Then every pixel is averaged over its samples.
template <int S, bool MS, bool SRGB, int CAP, bool GRAD>
__device__ __forceinline__ void resolve_bin(const FrameArgs &a, const uint2 *__restrict__ rec_a,
                                            const uint32_t *__restrict__ rec_m,
                                            const uint32_t *__restrict__ bstart, const uint32_t *__restrict__ bend,
                                            uint32_t *__restrict__ image, uint32_t *__restrict__ gx,
                                            const SmemTables &T, CellState<S / 8, CAP> &w, const int lane,
                                            const uint32_t b) {
    constexpr int MW = S / 8;
    // the bin's scene: viewport, first bin, image
    int W = a.W, H = a.H;
    uint32_t lb = b;
    int64_t image_off = 0;
    if (a.scenes != nullptr) {
        int lo = 0, hi = a.n_scenes - 1;  // last scene whose bin_off <= b
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (a.scenes[mid].bin_off <= b) lo = mid;
            else hi = mid - 1;
        }
        const SceneInfo *sc = a.scenes + lo;
        W = sc->W;
        H = sc->H;
        lb = b - sc->bin_off;
        image_off = sc->image_off;
        image += image_off;
    }
    // the bin: band `brow` of 64 >> sh cell rows, tile `tile` of 1 << sh
    // columns; lane l: cell l % cpr of the band's row l / cpr
    const int sh = a.bin_shift, cs = sh - 1, cpr = 1 << cs;  // cells per row: 1 << cs
    const int ntx = bin_cols(W, sh);
    const int brow = (int)(lb / ntx), tile = (int)(lb % ntx);
    const int tx0 = tile << sh;
    const int y0 = ((brow << (kBinShift - sh)) + (lane >> cs)) * 2;
    const int X0 = tx0 + 2 * (lane & (cpr - 1));  // this lane's cell: columns X0, X0 + 1, rows y0, y0 + 1
    // state: one white entry over every sample (multisample), or one colour
    // per pixel (single-sample output)
    int n = 1;
    uint32_t pc[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
    if constexpr (MS) {
#pragma unroll
        for (int k = 0; k <= MW; ++k) w.ent[0][k][lane] = 0xFFFFFFFFu;
    }
    const uint32_t beg = bstart[b], fin = bend[b];
    for (uint32_t base = beg; base < fin; base += kWin * 32) {
        __syncwarp();
        const int nb = (int)min((uint32_t)kWin, (fin - base + 31) / 32);  // batches in this window
        // the columns of the window's items (lane l: item 32 c + l of batch
        // c), all loads issued before the first is used
        uint32_t xws[kWin];
#pragma unroll
        for (int c = 0; c < kWin; ++c) {
            const uint32_t p = base + c * 32 + lane;
            xws[c] = c < nb && p < fin ? __ldg(&rec_a[p].y) : 0u;
        }
#pragma unroll
        for (int c = 0; c < kWin; ++c) {
            if (c >= nb) break;
            uint32_t cm = 0u;  // cells of this lane's item (a fragment: one cell of 2 columns)
            {
                const int x = (int)(xws[c] & 0xFFFFu);
                const int xb = min(x + (int)((xws[c] >> 16) & 0x1FFFu), W);
                cm = xb > x ? cell_bits((x - tx0) >> 1, (xb - tx0 + 1) >> 1, cpr, (int)(xws[c] >> 29)) : 0u;
            }
            // bit q of lane L's word: staged item q covers cell L (a transpose
            // of the 32 x 32 bit matrix of cell sets)
            uint32_t mine = 0u;
#pragma unroll
            for (int L = 0; L < 32; ++L) {
                const uint32_t bm = __ballot_sync(0xffffffffu, (cm >> L) & 1u);
                if (lane == L) mine = bm;
            }
            w.mine[c][lane] = mine;
        }
        __syncwarp();
        // this lane's items in draw order: batch cw, remaining bits
        int cw = 0;
        uint32_t bits = w.mine[0][lane];
        auto next_item = [&]() -> int {
            while (bits == 0u && ++cw < nb) bits = w.mine[cw][lane];
            if (bits == 0u) return -1;
            const int q = cw * 32 + __ffs(bits) - 1;
            bits &= bits - 1u;
            return q;
        };
        int q = next_item();
        uint32_t m[MW];
        uint2 r = make_uint2(0u, 0u);
        if (q >= 0) {
            r = __ldg(rec_a + base + q);
            load_mask<MW>(rec_m, base + q, m);
        }
        while (q >= 0) {
            const int qn = next_item();
            uint32_t mn[MW];
            uint2 rn = make_uint2(0u, 0u);
            if (qn >= 0) {
                rn = __ldg(rec_a + base + qn);
                load_mask<MW>(rec_m, base + qn, mn);
            }
            const uint32_t c = r.x;
            if (!GRAD || c - 1u >= a.n_grad) {  // a solid colour (else a gradient paint)
                const float sr = dec8<SRGB>(T, c & 0xFF, lane), sg = dec8<SRGB>(T, (c >> 8) & 0xFF, lane),
                            sb = dec8<SRGB>(T, (c >> 16) & 0xFF, lane), sa = lin8(c >> 24);
                if constexpr (MS) {
                    cell_apply<S, SRGB, CAP>(w, gx, lane, n, m, T, sr, sg, sb, sa);
                } else {
                    // single-sample output: alpha x coverage per pixel
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        int cov = 0;
#pragma unroll
                        for (int wd = 0; wd < MW; ++wd) cov += __popc(m[wd] & pixel_word_bits<S>(wd, k));
                        if (cov == 0) continue;
                        const float ak = sa * ((float)cov / (float)S);
                        pc[k] = blend_sample<SRGB>(T, lane, pc[k], sr, sg, sb, ak, 1.f - ak);
                    }
                }
            } else if constexpr (GRAD) {
                // a colour per pixel: one application per pixel
                const uint32_t xw = r.y;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int X = X0 + (k >> 1), Y = y0 + (k & 1);
                    uint32_t mk[MW];
                    int cov = 0;
#pragma unroll
                    for (int wd = 0; wd < MW; ++wd) {
                        mk[wd] = m[wd] & pixel_word_bits<S>(wd, k);
                        cov += __popc(mk[wd]);
                    }
                    if (cov == 0) continue;
                    const float4 gc = gradient_colour<SRGB>(a, T, c - 1u, (int)(int16_t)(xw & 0xFFFFu), (int)((xw >> 16) & 0x1FFFu),
                                                            X, Y, lane);
                    if constexpr (MS) {
                        cell_apply<S, SRGB, CAP>(w, gx, lane, n, mk, T, gc.x, gc.y, gc.z, gc.w);
                    } else {
                        const float ak = gc.w * ((float)cov / (float)S);
                        pc[k] = blend_sample<SRGB>(T, lane, pc[k], gc.x, gc.y, gc.z, ak, 1.f - ak);
                    }
                }
            }
            q = qn;
            r = rn;
#pragma unroll
            for (int k = 0; k < MW; ++k) m[k] = mn[k];
        }
    }
    __syncwarp();
    // per-pixel means: pixel k = px * 2 + py of the cell, at column X0 + px,
    // row y0 + py
    const double scale = 1.0 / (68719476736.0 * (double)(MS ? S : 1));
    uint32_t out[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        PixelSum p;
        if constexpr (MS) {
            for (int j = 0; j < n; ++j) {
                const uint32_t *ej = entry(w, gx, j, lane);
                int cov = 0;
#pragma unroll
                for (int wd = 0; wd < MW; ++wd) cov += __popc(ej[wd * 32] & pixel_word_bits<S>(wd, k));
                if (cov) add_sample<SRGB>(p, T, lane, ej[MW * 32], cov);
            }
        } else {
            add_sample<SRGB>(p, T, lane, pc[k], 1);
        }
        const int X = X0 + (k >> 1), Y = y0 + (k & 1);
        if (a.sums != nullptr) {  // a pass of a 256-sample frame: exact sums, encoded after the last pass
            if (X < W && Y < H) {
                longlong2 *q = reinterpret_cast<longlong2 *>(a.sums) + 2 * (image_off + (int64_t)Y * W + X);
                const longlong2 q0 = q[0], q1 = q[1];
                q[0] = make_longlong2(q0.x + p.r, q0.y + p.g);
                q[1] = make_longlong2(q1.x + p.b, q1.y + p.a);
            }
            continue;
        }
        out[k] = encode_mean<SRGB>(T, p, scale);
    }
    if (a.sums != nullptr) return;
#pragma unroll
    for (int py = 0; py < 2; ++py) {
        const int Y = y0 + py;
        if (Y >= H) continue;
        const int64_t pix = (int64_t)Y * W + X0;
        if (X0 + 1 < W && (reinterpret_cast<uintptr_t>(image + pix) & 7u) == 0) {
            *reinterpret_cast<uint2 *>(image + pix) = make_uint2(out[py], out[2 + py]);
        } else {
            if (X0 < W) image[pix] = out[py];
            if (X0 + 1 < W) image[pix + 1] = out[2 + py];
        }
    }
}

// Persistent resolve: each warp takes bins from the frame's bin queue until
// it is empty; a warp's overflow entry area is reused from bin to bin.
template <int S, bool MS, bool SRGB, bool GRAD>
__device__ __forceinline__ void resolve_persistent(const FrameArgs &a, const uint2 *__restrict__ rec_a,
                                                   const uint32_t *__restrict__ rec_m,
                                                   const uint32_t *__restrict__ bstart,
                                                   const uint32_t *__restrict__ bend, uint32_t *__restrict__ image,
                                                   uint32_t *__restrict__ overflow, uint32_t *__restrict__ bin_queue) {
    constexpr int CAP = MS ? kCellCap : 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemTables &T = *reinterpret_cast<SmemTables *>(smem_raw);
    {
        const ResolveTables *rt = a.rtables;
        if constexpr (SRGB)
            for (int i = threadIdx.x; i < 256 * 2; i += blockDim.x) T.dec8r[i] = rt->srgb_dec[i >> 1];
        for (int i = threadIdx.x; i < 256; i += blockDim.x) T.th[i] = rt->threshold[i];
        if constexpr (SRGB)
            for (int i = threadIdx.x; i < 1024; i += blockDim.x)
                reinterpret_cast<uint32_t *>(T.bin)[i] = reinterpret_cast<const uint32_t *>(rt->bin)[i];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    CellState<S / 8, CAP> &w = reinterpret_cast<CellState<S / 8, CAP> *>(smem_raw + sizeof(SmemTables))[warp];
    const int64_t slot = (int64_t)blockIdx.x * kResolveWarps + warp;
    // entries past CAP: up to one per sample of the cell
    uint32_t *gx = MS ? overflow + slot * (int64_t)(4 * S - CAP) * (S / 8 + 1) * 32 : nullptr;
    for (;;) {
        uint32_t b = 0;
        if (lane == 0) b = atomicAdd(bin_queue, 1u);
        b = __shfl_sync(0xffffffffu, b, 0);
        if ((int64_t)b >= a.n_bins) break;
        resolve_bin<S, MS, SRGB, CAP, GRAD>(a, rec_a, rec_m, bstart, bend, image, gx, T, w, lane, b);
        __syncwarp();
    }
}

template <int S, bool MS, bool SRGB>
__global__ void __launch_bounds__(kResolveWarps * 32, 4) k_resolve(FrameArgs a, const uint2 *__restrict__ rec_a,
                                                                 const uint32_t *__restrict__ rec_m,
                                                                 const uint32_t *__restrict__ bstart,
                                                                 const uint32_t *__restrict__ bend,
                                                                 uint32_t *__restrict__ image,
                                                                 uint32_t *__restrict__ overflow,
                                                                 uint32_t *__restrict__ bin_queue) {
    resolve_persistent<S, MS, SRGB, false>(a, rec_a, rec_m, bstart, bend, image, overflow, bin_queue);
}

// With gradient paints: registers capped so that two blocks stay resident
// (the per-pixel paint would otherwise take more).
template <int S, bool MS, bool SRGB>
__global__ void __launch_bounds__(kResolveWarps * 32, 2)
    k_resolve_grad(FrameArgs a, const uint2 *__restrict__ rec_a, const uint32_t *__restrict__ rec_m,
                   const uint32_t *__restrict__ bstart,
                   const uint32_t *__restrict__ bend, uint32_t *__restrict__ image, uint32_t *__restrict__ overflow,
                   uint32_t *__restrict__ bin_queue) {
    resolve_persistent<S, MS, SRGB, true>(a, rec_a, rec_m, bstart, bend, image, overflow, bin_queue);
}

// The image of a 256-sample frame from its passes' fixed-point sample sums
// (the same averaging and encoding as the resolve's last step).
template <bool SRGB>
__global__ void k_encode_sums(FrameArgs a, const long long *__restrict__ sums, uint32_t *__restrict__ image,
                              int64_t npix) {
    __shared__ SmemTables T;
    {
        const ResolveTables *rt = a.rtables;
        for (int i = threadIdx.x; i < 256; i += blockDim.x) T.th[i] = rt->threshold[i];
        if constexpr (SRGB)
            for (int i = threadIdx.x; i < 1024; i += blockDim.x)
                reinterpret_cast<uint32_t *>(T.bin)[i] = reinterpret_cast<const uint32_t *>(rt->bin)[i];
    }
    __syncthreads();
    const double scale = 1.0 / (68719476736.0 * 256.0);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x) {
        const longlong2 q0 = reinterpret_cast<const longlong2 *>(sums)[2 * i];
        const longlong2 q1 = reinterpret_cast<const longlong2 *>(sums)[2 * i + 1];
        const float ar = (float)((double)q0.x * scale), ag = (float)((double)q0.y * scale);
        const float ab = (float)((double)q1.x * scale), aa = (float)((double)q1.y * scale);
        image[i] = enc8<SRGB>(T, ar) | (enc8<SRGB>(T, ag) << 8) | (enc8<SRGB>(T, ab) << 16) | (enc_lin(aa) << 24);
    }
}

// Exhaustive check of enc_srgb against the definition (the number of
// thresholds <= the clamped value, by binary search) over every float bit
// pattern in [lo, hi).
__global__ void k_selftest_encode(const ResolveTables *__restrict__ rt, uint32_t lo, uint32_t hi,
                                  unsigned long long *__restrict__ bad) {
    __shared__ SmemTables T;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) T.th[i] = rt->threshold[i];
    for (int i = threadIdx.x; i < 4096; i += blockDim.x) T.bin[i] = rt->bin[i];
    __syncthreads();
    unsigned long long local = 0;
    for (uint64_t u = lo + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < hi;
         u += (uint64_t)gridDim.x * blockDim.x) {
        const float v = __uint_as_float((uint32_t)u);
        const float c = fmin_r(fmax_r(v, 0.f), 1.f);
        int a = 0, b = 255;  // thresholds th[0..254] ascending: count those <= c
        while (a < b) {
            const int m = (a + b) >> 1;
            if (T.th[m] <= c) a = m + 1;
            else b = m;
        }
        if (enc_srgb(T, v) != (uint32_t)a) ++local;
    }
    if (local) atomicAdd(bad, local);
}

// ---------------------------------------------------- scene upload --
// Checks of spr_validate_scene and unifyCurveVertexOrder (ras_base.cpp:523-569)
// on the device.  flags: bit 0 = invalid scene, bit 1 = vertex ranges of
// consecutive curves not disjoint and ascending (the in-place reversal would
// depend on the curve order: the host path handles such scenes).
__global__ void k_scene_vertices(const uint32_t *__restrict__ vpid, uint32_t V, uint32_t P,
                                 uint32_t *__restrict__ vmap, uint32_t *__restrict__ flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    vmap[i] = i;
    if (vpid[i] >= P) atomicOr(flags, 1u);
}

__global__ void k_scene_curves(const uint32_t *__restrict__ cvp, const uint8_t *__restrict__ ctype,
                               const uint32_t *__restrict__ cpid, const float *__restrict__ arcw, uint32_t C,
                               uint32_t V, uint32_t P, float2 *__restrict__ vert, uint32_t *__restrict__ vmap,
                               CurveDesc *__restrict__ cd, uint32_t *__restrict__ flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C) return;
    const int type = ctype[i];
    const bool known = type == kLinear || type == kQuad || type == kCubic || type == kRational;
    const int vn = type & 7;
    const uint32_t p = cvp[i], pid = cpid[i];
    bool bad = !known || (type == kRational && arcw == nullptr) || (uint64_t)p + (uint64_t)vn > V || pid >= P ||
               (i > 0 && pid < cpid[i - 1]);
    if (bad) {
        atomicOr(flags, 1u);
        return;
    }
    if (i + 1 < C && (uint64_t)p + (uint64_t)vn > (uint64_t)cvp[i + 1]) atomicOr(flags, 2u);
    // reverse unless (y_first, x_first) < (y_last, x_last) as float bit patterns
    const float2 vf = vert[p], vl = vert[p + vn - 1];
    const uint32_t bxf = __float_as_uint(vf.x), byf = __float_as_uint(vf.y);
    const uint32_t bxl = __float_as_uint(vl.x), byl = __float_as_uint(vl.y);
    const uint32_t rev = (byf < byl || (byf == byl && bxf < bxl)) ? 0u : 1u;
    CurveDesc d;
    d.vpos = p;
    d.pid = pid;
    d.w = type == kRational ? arcw[i] : 0.f;
    d.type = (uint32_t)type | (rev << 8);
    cd[i] = d;
    if (rev) {
        for (int k = 0; k < vn / 2; ++k) {
            const float2 t = vert[p + k];
            vert[p + k] = vert[p + vn - 1 - k];
            vert[p + vn - 1 - k] = t;
        }
        for (int k = 0; k < vn; ++k) vmap[p + k] = p + vn - 1 - k;
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


int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
    }
    return n;
}

// Shared memory of a resolve block: the tables and one cell state per warp.
size_t resolve_smem(int S, bool ms) {
    const int MW = S / 8, CAP = ms ? kCellCap : 1;
    return sizeof(SmemTables) + (size_t)kResolveWarps * ((size_t)CAP * (MW + 1) * 32 * 4 + (size_t)kWin * 32 * 4);
}

// Resolve blocks per SM: as many as fit in shared memory (at most 4), or
// the tuned count if lower.
int resolve_bps(const FrameArgs &a) {
    const int fit = std::max(1, std::min<int>(kResolveMaxBlocksPerSM, (int)((227u << 10) / resolve_smem(a.S, a.ms_output))));
    return a.resolve_bps >= 1 && a.resolve_bps < fit ? a.resolve_bps : fit;
}

int64_t resolve_blocks(const FrameArgs &a) {
    const int64_t need = (a.n_bins + kResolveWarps - 1) / kResolveWarps;
    return std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)sm_count() * resolve_bps(a)));
}

template <int S, bool MS, bool SRGB, bool GRAD>
void resolve_variant_g(const FrameArgs &a, const uint2 *rec_a, const uint32_t *rec_m, const uint32_t *bstart, const uint32_t *bend, uint32_t *image, uint32_t *overflow,
                     uint32_t *queue, cudaStream_t s) {
    constexpr int CAP = MS ? kCellCap : 1;
    const size_t smem = sizeof(SmemTables) + (size_t)kResolveWarps * sizeof(CellState<S / 8, CAP>);
    auto kern = GRAD ? k_resolve_grad<S, MS, SRGB> : k_resolve<S, MS, SRGB>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    // resident blocks per SM (registers or shared memory), so that every
    // launched block runs at once; never more than resolve_blocks(a), which
    // sized the overflow entry area
    int fit = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, kResolveWarps * 32, smem) != cudaSuccess || fit < 1)
        fit = 1;
    const int64_t blocks = std::min<int64_t>(resolve_blocks(a), (int64_t)sm_count() * fit);
    kern<<<(unsigned)blocks, kResolveWarps * 32, smem, s>>>(a, rec_a, rec_m, bstart, bend, image, overflow, queue);
}

// Gradient paints get their own instantiations: the per-pixel paint costs
// registers that plain frames should not pay for.
template <int S, bool MS, bool SRGB>
void resolve_variant(const FrameArgs &a, const uint2 *rec_a, const uint32_t *rec_m, const uint32_t *bstart, const uint32_t *bend, uint32_t *image, uint32_t *overflow,
                     uint32_t *queue, cudaStream_t s) {
    if (a.grad_table != nullptr)
        resolve_variant_g<S, MS, SRGB, true>(a, rec_a, rec_m, bstart, bend, image, overflow, queue, s);
    else
        resolve_variant_g<S, MS, SRGB, false>(a, rec_a, rec_m, bstart, bend, image, overflow, queue, s);
}

}  // namespace

int launch_transform(const FrameArgs &a, float2 *tvert, uint32_t *path_flags, uint8_t *path_visible, cudaStream_t s) {
    cudaMemsetAsync(path_flags, 0, sizeof(uint32_t) * (size_t)a.P, s);
    int n = 0;
    if (a.V > 0) k_transform<<<grid_for(a.V), kThreads, 0, s>>>(a, tvert, path_flags), ++n;
    if (a.P > 0) k_path_visible<<<grid_for(a.P), kThreads, 0, s>>>(a.P, path_flags, path_visible), ++n;
    return n;
}

int launch_curve_count(const FrameArgs &a, const float2 *tvert, const uint8_t *vis, uint32_t *counts, cudaStream_t s) {
    if (a.C <= 0) return 0;
    k_curve_count<<<grid_for(a.C), kThreads, 0, s>>>(a, tvert, vis, counts);
    return 1;
}

int launch_emit_keys(const FrameArgs &a, const uint32_t *counts, uint32_t *key, uint32_t *val, cudaStream_t s) {
    if (a.C <= 0) return 0;
    k_emit_keys<<<grid_for(a.C), kThreads, 0, s>>>(a, counts, key, val);
    return 1;
}

int launch_curve_emit(const FrameArgs &a, const float2 *tvert, const uint8_t *vis, const uint32_t *offsets,
                       const uint32_t *order, int2 *entries, const FrameCounters *ctr, cudaStream_t s) {
    if (a.C <= 0) return 0;
    k_curve_emit<<<grid_for(a.C, kEmitWarps * 32), kEmitWarps * 32, 0, s>>>(a, tvert, vis, offsets, order, entries,
                                                                           ctr);
    return 1;
}

int launch_fragment(const FrameArgs &a, const float2 *tvert, const int2 *entries, int64_t cap_nf,
                    const FrameCounters *ctr, int32_t *key, uint32_t *pidw, int8_t *wn, uint32_t *mask,
                    uint64_t *sort_key, uint32_t *sort_val, cudaStream_t s) {
    if (cap_nf <= 0) return 0;
    const unsigned g = grid_for(cap_nf);
    if (a.S == 8)
        k_fragment<8><<<g, kThreads, 0, s>>>(a, tvert, entries, ctr, key, pidw, wn, mask, sort_key, sort_val);
    else if (a.S == 16)
        k_fragment<16><<<g, kThreads, 0, s>>>(a, tvert, entries, ctr, key, pidw, wn, mask, sort_key, sort_val);
    else
        k_fragment<32><<<g, kThreads, 0, s>>>(a, tvert, entries, ctr, key, pidw, wn, mask, sort_key, sort_val);
    return 1;
}

int64_t scan_mark_status_words(int64_t cap_nf) { return 2 * std::max<int64_t>(1, (cap_nf + kMarkTile - 1) / kMarkTile); }

int launch_scan_mark(const FrameArgs &a, int64_t cap_nf, const uint64_t *skey, int8_t *wn_scan, int4 *draw, uint32_t *heads, uint32_t *item_scene, uint32_t *bin_count,
                     FrameCounters *counters, uint64_t *tile_status, uint32_t spin_cap, cudaStream_t s) {
    const int64_t words = scan_mark_status_words(cap_nf);
    k_scan_mark<<<(unsigned)(words / 2), kMarkThreads, 0, s>>>(a, skey, wn_scan, draw, heads, item_scene,
                                                               bin_count, counters, tile_status, tile_status + words / 2,
                                                               spin_cap);
    return 1;
}

int launch_stencil(const FrameArgs &a, int64_t cap_nf, FrameCounters *ctr, const uint64_t *skey, const uint32_t *perm,
                   const uint32_t *mask, const int8_t *wn_scan, const uint32_t *heads, uint32_t *merged,
                   uint32_t spin_cap, cudaStream_t s) {
    if (cap_nf <= 0) return 0;
    const unsigned g = grid_for(cap_nf);
    if (a.S == 8)
        k_stencil<8><<<g, kThreads, 0, s>>>(a, ctr, skey, perm, mask, wn_scan, heads, merged, spin_cap);
    else if (a.S == 16)
        k_stencil<16><<<g, kThreads, 0, s>>>(a, ctr, skey, perm, mask, wn_scan, heads, merged, spin_cap);
    else
        k_stencil<32><<<g, kThreads, 0, s>>>(a, ctr, skey, perm, mask, wn_scan, heads, merged, spin_cap);
    return 1;
}

int launch_bin_scatter(const FrameArgs &a, const int4 *draw, const uint32_t *item_scene, int64_t cap_items,
                       const FrameCounters *ctr, const uint32_t *bin_off, uint32_t *bin_fill, uint32_t *pval,
                       cudaStream_t s) {
    if (cap_items <= 0) return 0;
    k_bin_scatter<<<grid_for(cap_items), kThreads, 0, s>>>(a, draw, item_scene, ctr, bin_off, bin_fill, pval);
    return 1;
}

int launch_bin_count(const FrameArgs &a, const int4 *draw, const uint32_t *item_scene, int64_t cap_items,
                     const FrameCounters *ctr, uint32_t *bin_count, cudaStream_t s) {
    if (cap_items <= 0) return 0;
    k_bin_count<<<grid_for(cap_items), kThreads, 0, s>>>(a, draw, item_scene, ctr, bin_count);
    return 1;
}

int launch_bin_sort(const uint32_t *bin_off, int64_t nbins, uint32_t *pval, const FrameCounters *ctr, int S,
                    int bin_shift, const int4 *draw, const uint32_t *merged, uint2 *rec_a, uint32_t *rec_m,
                    cudaStream_t s) {
    const int band_mask = (1 << (kBinShift - bin_shift)) - 1;  // cell rows per band - 1
    if (nbins <= 0) return 0;
    const unsigned g = (unsigned)((nbins + kBinSortWarps - 1) / kBinSortWarps);
    if (S == 8)
        k_bin_sort<1><<<g, kBinSortWarps * 32, 0, s>>>(bin_off, nbins, pval, ctr, draw, merged, rec_a, rec_m, band_mask);
    else if (S == 16)
        k_bin_sort<2><<<g, kBinSortWarps * 32, 0, s>>>(bin_off, nbins, pval, ctr, draw, merged, rec_a,
                                                        reinterpret_cast<uint2 *>(rec_m), band_mask);
    else
        k_bin_sort<4><<<g, kBinSortWarps * 32, 0, s>>>(bin_off, nbins, pval, ctr, draw, merged, rec_a,
                                                        reinterpret_cast<uint4 *>(rec_m), band_mask);
    return 1;
}


int launch_resolve(const FrameArgs &a, const uint2 *rec_a, const uint32_t *rec_m, const uint32_t *bstart, const uint32_t *bend, uint32_t *image, uint32_t *overflow,
                    FrameCounters *counters, cudaStream_t s) {
    if (a.n_bins <= 0) return 0;
    uint32_t *queue = &counters->bin_queue;
    cudaMemsetAsync(queue, 0, sizeof(uint32_t), s);
    const bool ms = a.ms_output != 0, srgb = a.srgb != 0;
    if (a.S == 8) {
        if (ms && srgb) resolve_variant<8, true, true>(a, rec_a, rec_m, bstart, bend, image, overflow, queue, s);
        else if (ms) resolve_variant<8, true, false>(a, rec_a, rec_m, bstart, bend, image, overflow, queue, s);
        else if (srgb) resolve_variant<8, false, true>(a, rec_a, rec_m, bstart, bend, image, overflow, queue, s);
        else resolve_variant<8, false, false>(a, rec_a, rec_m, bstart, bend, image, overflow, queue, s);
    } else if (a.S == 16) {
        if (ms && srgb) resolve_variant<16, true, true>(a, rec_a, rec_m, bstart, bend, image, overflow, queue, s);
        else if (ms) resolve_variant<16, true, false>(a, rec_a, rec_m, bstart, bend, image, overflow, queue, s);
        else if (srgb) resolve_variant<16, false, true>(a, rec_a, rec_m, bstart, bend, image, overflow, queue, s);
        else resolve_variant<16, false, false>(a, rec_a, rec_m, bstart, bend, image, overflow, queue, s);
    } else {
        if (ms && srgb) resolve_variant<32, true, true>(a, rec_a, rec_m, bstart, bend, image, overflow, queue, s);
        else if (ms) resolve_variant<32, true, false>(a, rec_a, rec_m, bstart, bend, image, overflow, queue, s);
        else if (srgb) resolve_variant<32, false, true>(a, rec_a, rec_m, bstart, bend, image, overflow, queue, s);
        else resolve_variant<32, false, false>(a, rec_a, rec_m, bstart, bend, image, overflow, queue, s);
    }
    return 1;
}

int launch_encode_sums(const FrameArgs &a, const long long *sums, uint32_t *image, int64_t npix, cudaStream_t s) {
    if (npix <= 0) return 0;
    const unsigned grid = (unsigned)std::min<int64_t>((npix + 255) / 256, 152 * 8);
    if (a.srgb) k_encode_sums<true><<<grid, 256, 0, s>>>(a, sums, image, npix);
    else k_encode_sums<false><<<grid, 256, 0, s>>>(a, sums, image, npix);
    return 1;
}

// The output view (drawOutputResize with output_scale.{vert,frag}.glsl,
// ras_base.cpp:760-803): pixel (x, y) shows the image texel nearest to
// inv * (x + 0.5, y + 0.5, 0, 1) after the divide by w, clamped to the edge
// (the scale texture's GL_NEAREST / GL_CLAMP_TO_EDGE).  inv holds the
// inverse transform's rows 0, 1 and 3, columns 0, 1 and 3.
__global__ void k_output_view(const uint32_t *__restrict__ image, uint32_t *__restrict__ out, int W, int H,
                              OutputInverse inv) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)W * H) return;
    const int x = (int)(i % W), y = (int)(i / W);
    const float px = (float)x + 0.5f, py = (float)y + 0.5f;
    const float qx = inv.m[0] * px + inv.m[1] * py + inv.m[2];
    const float qy = inv.m[3] * px + inv.m[4] * py + inv.m[5];
    const float qw = inv.m[6] * px + inv.m[7] * py + inv.m[8];
    float u = qx / qw, v = qy / qw;
    u = fminf(fmaxf(floorf(u), 0.f), (float)(W - 1));  // fmaxf takes 0 for a NaN
    v = fminf(fmaxf(floorf(v), 0.f), (float)(H - 1));
    out[i] = image[(int64_t)(int)v * W + (int)u];
}

int launch_output_view(const uint32_t *image, uint32_t *out, int W, int H, const OutputInverse &inv, cudaStream_t s) {
    const int64_t n = (int64_t)W * H;
    if (n <= 0) return 0;
    k_output_view<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(image, out, W, H, inv);
    return 1;
}

int launch_selftest_encode(const ResolveTables *rt, unsigned long long *bad, cudaStream_t s) {
    // non-negative floats up to and a little beyond 1.0, plus the negative zero
    k_selftest_encode<<<4 * 152, 256, 0, s>>>(rt, 0u, 0x3F800100u, bad);
    k_selftest_encode<<<1, 256, 0, s>>>(rt, 0x80000000u, 0x80000100u, bad);
    return 2;
}

int64_t resolve_warps(const FrameArgs &a) { return resolve_blocks(a) * kResolveWarps; }

int64_t resolve_overflow_words(const FrameArgs &a) {
    if (!a.ms_output) return 0;
    const int S = a.S == 256 ? 32 : a.S;
    return resolve_warps(a) * (int64_t)(4 * S - kCellCap) * (S / 8 + 1) * 32;
}

int launch_scene_prepare(const uint32_t *cvp, const uint8_t *ctype, const uint32_t *cpid, const float *arcw,
                         uint32_t C, uint32_t V, uint32_t P, float2 *vert, const uint32_t *vpid, uint32_t *vmap,
                         CurveDesc *cd, uint32_t *flags, cudaStream_t s) {
    int n = 0;
    if (V > 0) k_scene_vertices<<<grid_for(V), kThreads, 0, s>>>(vpid, V, P, vmap, flags), ++n;
    if (C > 0) k_scene_curves<<<grid_for(C), kThreads, 0, s>>>(cvp, ctype, cpid, arcw, C, V, P, vert, vmap, cd, flags), ++n;
    return n;
}

int launch_fill(uint32_t *image, int64_t n, uint32_t value, cudaStream_t s) {
    if (n <= 0) return 0;
    k_fill<<<grid_for(n), kThreads, 0, s>>>(image, n, value);
    return 1;
}

int launch_decode_keys(const uint64_t *skey, int64_t n, int nrows, int32_t *out, cudaStream_t s) {
    if (n <= 0) return 0;
    k_decode_keys<<<grid_for(n), kThreads, 0, s>>>(skey, n, nrows, out);
    return 1;
}

}  // namespace spr
