// spr_api.cpp -- the C ABI of include/spr.h: handle lifetime, scene upload
// (addVg + unifyCurveVertexOrder), per-frame orchestration of the CUDA
// stages (rasterizeImpl), read-back, PNG output, element counts, step timing
// and stage dumps.
//
// Device memory: the scene lives in per-handle buffers written once by
// spr_set_scene; every per-frame array is a grow-only buffer of the handle
// (the role of the reference's 256 MB bump arena, cuda_cached_allocator.h),
// so steady-state frames allocate nothing.  The frame reads back three
// counts to size its work (fragments, merged fragments + spans, resolve
// pairs); everything else stays on the device.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/spr.h"
#include "spr_internal.h"

namespace spr {
int write_png_rgba(const char *path, const uint8_t *rgba, int w, int h);
}

using namespace spr;

namespace {

// Device bytes held by one handle's buffers and the caller's cap on them
// (0 = none; spr_set_memory_limit), the counterpart of the reference's fixed
// arena that throws when it is exhausted (cuda_cached_allocator.h:77-82).
struct Budget {
    size_t used = 0;
    size_t limit = 0;
};

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    Budget *budget = nullptr;  // the owning handle's, if any
    void release() {
        if (p) cudaFree(p);
        if (budget) budget->used -= bytes;
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T *as() const {
        return static_cast<T *>(p);
    }
};

// Bumped whenever a buffer is reallocated: a captured frame graph holds the
// buffer addresses of its capture and is replayed only while this is unchanged.
std::atomic<uint64_t> g_alloc_gen{0};

int ensure(DevBuf &b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return SPR_OK;
    size_t want = bytes + bytes / 4;
    want = (want + 255) & ~(size_t)255;
    if (b.budget && b.budget->limit) {
        // over the cap even at the exact size: refuse, keeping the old buffer
        const size_t others = b.budget->used - b.bytes;
        const size_t exact = (bytes + 255) & ~(size_t)255;
        if (others + exact > b.budget->limit) return SPR_ERR_OUT_OF_MEMORY;
        want = std::min(want, b.budget->limit - others);
    }
    g_alloc_gen.fetch_add(1);
    b.release();
    if (cudaMalloc(&b.p, want) != cudaSuccess) {
        cudaGetLastError();
        b.p = nullptr;
        return SPR_ERR_OUT_OF_MEMORY;
    }
    b.bytes = want;
    if (b.budget) b.budget->used += want;
    return SPR_OK;
}

int cuda_status() {
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return SPR_OK;
    if (e == cudaErrorMemoryAllocation) return SPR_ERR_OUT_OF_MEMORY;
    return SPR_ERR_CUDA;
}

int bits_for(uint64_t v) {  // number of bits needed to hold values 0..v
    int b = 0;
    while (v) {
        ++b;
        v >>= 1;
    }
    return b;
}

const char *kStepNames[] = {"transform", "intersect_count", "intersect_emit_fragment", "sort", "scan_mark",
                            "stencil",   "resolve_bin",     "resolve"};
constexpr int kSteps = 8;

}  // namespace

struct spr_handle {
    spr_config cfg{};
    float m[16];
    // tables
    DevBuf mask_table;
    int table_samples = 0;
    DevBuf rtables;
    // scene
    bool has_scene = false;
    uint32_t P = 0, C = 0, V = 0;
    DevBuf vertex, vpid, curves, rule, fill, affine;
    bool has_affine = false;
    // batch frames (n_scenes > 0): per-scene viewports/transforms/images and
    // the scene of every path; single-scene frames use cfg and m
    int n_scenes = 0;
    std::vector<SceneInfo> scenes_h;
    int scenes_shift = kBinShift;  // bin geometry of the scene table on the device
    DevBuf scenes_d, path_scene, item_scene;
    // differentiable frames: per-fragment chords and left masks, per-item
    // paths, the per-block tapes, the transformed-vertex gradient and the
    // stored -> input vertex map
    DevBuf chord, lmask, vmask, item_path, tape, tape_rec, grad_tvert, vmap, bitems, chain, ekey[2], eval[2];
    // 256-sample frames: the pass being rendered, the passes' fixed-point
    // sample sums, and a pass's fill gradient / the summed vertex gradient
    int pass = 0;
    DevBuf sums, gfill_pass, gtvert_total;
    // gradient paints: table entries and ramp texels on the device, and the
    // reverse transform (pixel -> scene) of their coordinates
    DevBuf grad_table, grad_ramp;
    DevBuf path_start;  // first curve of every path (the per-path segment sort)
    // launch choices (spr_autotune; -1 / 0 = the built-in rule): fragment
    // sort (0 device-wide radix, 1 per-path segments), curve-emission order
    // (0 off, 1 on), resolve blocks per SM
    int tune_sort = -1, tune_emit = -1, tune_bps = 0, tune_bin_w = 0;
    int auto_bin_shift = kBinShift;  // the built-in tile, from the last sized frame's spans
    uint32_t n_grad = 0;
    float rev[13] = {1.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 1.f};
    // output view (setOutputTransform / enableOutputTransform): the inverse
    // transform's rows 0, 1, 3 and the view's buffer
    bool out_tf = false;
    OutputInverse out_inv{{1.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 1.f}};
    DevBuf output;
    // raw curve arrays of the device-side scene upload (kept for vertex updates)
    DevBuf sc_vpos, sc_type, sc_pid, sc_w, scene_flags;
    bool scene_on_device = false, scene_has_arcw = false;
    int tape_depth = 128;
    // frame buffers
    DevBuf tvert, pflags, pvis, counts, offsets, scan_tmp, entries, key, pidw, wn, mask, skey[2], sval[2], sort_tmp,
        wn_scan, draw, heads, merged, pval, rec_a, rec_m, bins, image, counters, dump_tmp, overflow;
    // look-back tile words of the frame's scans: entry offsets, scan-mark, pair offsets
    DevBuf lb_off, lb_mark, lb_pair;
    uint64_t *skey_sorted = nullptr;
    uint32_t *perm_sorted = nullptr;
    const uint32_t *pv_sorted = nullptr;  // resolve pairs in bin order
    // the buffers hold a differentiable forward frame of the current inputs:
    // a backward needs no new geometry pass
    bool diff_ready = false;
    // host staging
    FrameCounters *h_counters = nullptr;
    uint32_t *h_u32 = nullptr;
    // last frame
    spr_element_number en{};
    int64_t nf = 0, nm = 0, ns = 0, npairs = 0;
    bool frame_valid = false;
    int launches = 0, host_syncs = 0;
    int frame_W = 0, frame_H = 0, frame_S = 8;
    // Buffer capacities of the frame (intersection entries, draw items,
    // resolve pairs).  A "sized" frame reads its sizes back as it goes and
    // sets them with headroom; while they hold (caps_ok), frames run without
    // host reads, taking their sizes from the device counters, and a frame
    // whose sizes outgrow them is rendered again (sized) before anything
    // reads it.
    int64_t cap_nf = 0, cap_items = 0, cap_pairs = 0;
    bool caps_ok = false;
    // a frame rendered without host reads whose counters have not been read
    // yet (their copy in h_counters is complete once done_ev is); stale:
    // the inputs changed after it was enqueued (it cannot be rendered again)
    bool pending = false, pending_stale = false;
    cudaStream_t pending_stream = nullptr;
    cudaEvent_t done_ev = nullptr;
    // bounded waits of the look-back scans: polls before giving up, and (for
    // tests of the timeout) a tile of the entry-offset scan that never
    // publishes (-1: none)
    uint32_t lb_spin_cap = kLbSpinCap;
    int64_t lb_hold_tile = -1;
    // graph replay of unchanged frames: the launch sequence of a frame
    // rendered without host reads, captured once (it depends on the
    // capacities, not on the sizes)
    bool graph_mode = false, capturing = false, graph_failed = false;
    cudaGraphExec_t gexec = nullptr;
    uint64_t gexec_gen = 0;
    cudaStream_t cap_stream = nullptr;
    int graph_replays = 0;
    // timing
    bool timing = false;
    cudaEvent_t ev[kSteps + 1] = {};
    double step_ms[kSteps] = {};
    Budget budget;
};

namespace {

// Every device buffer of a handle.
std::vector<DevBuf *> handle_bufs(spr_handle *h) {
    return {&h->mask_table, &h->rtables, &h->vertex,   &h->vpid,      &h->curves,  &h->rule,
                      &h->fill,       &h->affine,  &h->tvert,    &h->pflags,    &h->pvis,    &h->counts,
                      &h->offsets,    &h->scan_tmp, &h->entries, &h->key,       &h->pidw,    &h->wn,
                      &h->mask,       &h->skey[0], &h->skey[1],  &h->sval[0],   &h->sval[1], &h->sort_tmp,
                      &h->wn_scan,    &h->draw,    &h->heads,    &h->lb_off,    &h->merged,  &h->pval,
                      &h->rec_a,      &h->rec_m,   &h->bins,
                      &h->image,      &h->counters, &h->dump_tmp, &h->overflow, &h->scenes_d, &h->path_scene,
                      &h->item_scene, &h->chord,  &h->lmask,   &h->item_path, &h->tape,  &h->tape_rec,
                      &h->grad_tvert, &h->vmap, &h->bitems, &h->vmask, &h->chain, &h->ekey[0], &h->ekey[1], &h->eval[0],
                      &h->eval[1], &h->sc_vpos, &h->sc_type, &h->sc_pid, &h->sc_w, &h->scene_flags,
                      &h->sums, &h->gfill_pass, &h->gtvert_total, &h->grad_table, &h->grad_ramp, &h->path_start,
                      &h->output, &h->lb_mark, &h->lb_pair};
}

}  // namespace

namespace {

void drop_graph(spr_handle *h, bool inputs_changed = true) {
    if (inputs_changed) {
        h->diff_ready = false;
        if (h->pending) h->pending_stale = true;
    }
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
    h->graph_failed = false;
}

int validate_config(const spr_config *c) {
    if (c->width < 1 || c->height < 1 || c->width > 4096 || c->height > 4096) return SPR_ERR_INVALID_ARG;
    if (c->samples != 8 && c->samples != 16 && c->samples != 32 && c->samples != 256) return SPR_ERR_INVALID_ARG;
    // 256 samples are resolved per sample only: the coverage-as-alpha output
    // needs every sample of an item at once, which the passes do not have
    if (c->samples == 256 && !c->ms_output) return SPR_ERR_INVALID_ARG;
    return SPR_OK;
}

int build_tables(spr_handle *h) {
    if (h->table_samples == h->cfg.samples) return SPR_OK;
    const bool passes = h->cfg.samples == 256;
    const int words = passes ? 4 : h->cfg.samples / 8;
    std::vector<uint32_t> t((size_t)65536 * words * (passes ? kPasses256 : 1));
    if (passes) {
        for (int g = 0; g < kPasses256; ++g) build_pass_mask_table_256(g, t.data() + (size_t)g * 65536 * 4);
    } else {
        build_mask_table(h->cfg.samples, t.data());
    }
    int st = ensure(h->mask_table, t.size() * 4);
    if (st) return st;
    if (cudaMemcpy(h->mask_table.p, t.data(), t.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) return cuda_status();
    h->table_samples = h->cfg.samples;
    return SPR_OK;
}

// Bin geometry of a frame (shift: tiles of 1 << shift columns).
int frame_bin_shift(const spr_handle *h, bool diff) {
    if (diff) return kBinShift;
    switch (h->tune_bin_w) {
    case 8: return 3;
    case 16: return 4;
    case 32: return 5;
    case 64: return 6;
    default: return h->auto_bin_shift;
    }
}

FrameArgs make_args(const spr_handle *h, bool diff = false) {
    FrameArgs a;
    a.W = h->cfg.width;
    a.H = h->cfg.height;
    a.S = h->cfg.samples;
    a.ms_output = h->cfg.ms_output;
    a.srgb = h->cfg.srgb;
    a.P = (int)h->P;
    a.C = (int)h->C;
    a.V = (int)h->V;
    std::memcpy(a.m, h->m, sizeof(a.m));
    a.vertex = h->vertex.as<float2>();
    a.vertex_pid = h->vpid.as<uint32_t>();
    a.affine = h->has_affine ? h->affine.as<float>() : nullptr;
    a.curves = h->curves.as<CurveDesc>();
    a.fill_rule = h->rule.as<uint8_t>();
    a.fill_rgba = h->fill.as<uint32_t>();
    a.mask_table = h->mask_table.as<uint32_t>();
    a.rtables = h->rtables.as<ResolveTables>();
    a.chord = nullptr;
    a.lmask = nullptr;
    a.vmask = nullptr;
    a.item_path = nullptr;
    a.pass_dy = 0.f;
    a.sums = nullptr;
    a.grad_table = h->n_grad ? h->grad_table.as<float4>() : nullptr;
    a.n_grad = h->n_grad;
    a.grad_ramp = h->grad_ramp.as<uint32_t>();
    std::memcpy(a.rev, h->rev, sizeof(a.rev));
    a.resolve_bps = h->tune_bps;
    if (h->cfg.samples == 256) {  // the current pass of 32 samples
        a.S = 32;
        a.pass_dy = pass_shift_256(h->pass);
        a.mask_table += (size_t)h->pass * 65536 * 4;
        a.sums = h->sums.as<long long>();
    }
    if (h->n_scenes > 0) {
        a.path_scene = h->path_scene.as<uint32_t>();
        a.scenes = h->scenes_d.as<SceneInfo>();
        a.n_scenes = h->n_scenes;
        const SceneInfo &last = h->scenes_h.back();
        a.n_bins = (int64_t)last.bin_off + (int64_t)last.ntx * last.nrows;
        a.bin_shift = h->scenes_shift;
        a.alt_shift = !diff && h->tune_bin_w == 0 ? kPlainBinShift + kBinShift - a.bin_shift : -1;
    } else {
        a.path_scene = nullptr;
        a.scenes = nullptr;
        a.n_scenes = 0;
        a.bin_shift = frame_bin_shift(h, diff);
        a.alt_shift = !diff && h->tune_bin_w == 0 ? kPlainBinShift + kBinShift - a.bin_shift : -1;
        a.n_bins = (int64_t)bin_cols(a.W, a.bin_shift) * bin_rows(a.H, a.bin_shift);
    }
    return a;
}

// Pixels of the frame's image buffer (all scenes of a batch).
int64_t frame_pixels(const spr_handle *h) {
    if (h->n_scenes > 0) {
        const SceneInfo &last = h->scenes_h.back();
        return last.image_off + (int64_t)last.W * last.H;
    }
    return (int64_t)h->cfg.width * h->cfg.height;
}

// The view's pointers and sizes (the element checks follow in validate_scene
// on the host, or in k_scene_vertices / k_scene_curves on the device).
int validate_view(const spr_scene_view *v) {
    if (!v) return SPR_ERR_INVALID_ARG;
    if ((v->n_vertices && (!v->vertex || !v->vertex_path_id)) ||
        (v->n_curves && (!v->curve_vertex_pos || !v->curve_type || !v->curve_path_id)) ||
        (v->n_paths && (!v->path_fill_rule || !v->path_fill_rgba)))
        return SPR_ERR_INVALID_ARG;
    if (v->n_vertices > (1u << 30) || v->n_curves > (1u << 30) || v->n_paths > (1u << 30))
        return SPR_ERR_INVALID_SCENE;
    return SPR_OK;
}

// A gradient table and ramp as spr_set_gradients takes them: the ramp in
// whole 1024-texel rows, every entry's ramp run inside one row.
int check_gradients(const uint32_t *table, uint32_t n_entries, const uint32_t *ramp, uint32_t n_texels) {
    if (!table || !ramp || n_texels == 0 || n_texels % 1024 != 0 || n_entries > 0x01000000u)
        return SPR_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < n_entries; ++i) {
        const int32_t p = (int32_t)table[12 * i + 6];
        float scale;
        std::memcpy(&scale, &table[12 * i + 7], 4);
        const float n1 = scale * 1024.f;  // ramp length - 1
        if (!(n1 >= 0.f)) continue;       // solid slot: never sampled
        if (p < 0 || (uint64_t)p + (uint64_t)n1 >= n_texels || (p & 1023) + (int64_t)n1 > 1023)
            return SPR_ERR_INVALID_ARG;
    }
    return SPR_OK;
}

int validate_scene(const spr_scene_view *v) {
    int st = validate_view(v);
    if (st) return st;
    uint32_t last = 0;
    for (uint32_t i = 0; i < v->n_curves; ++i) {
        const int t = v->curve_type[i];
        if (t != SPR_CURVE_LINEAR && t != SPR_CURVE_QUADRATIC && t != SPR_CURVE_CUBIC && t != SPR_CURVE_RATIONAL)
            return SPR_ERR_INVALID_SCENE;
        if (t == SPR_CURVE_RATIONAL && !v->curve_arc_w) return SPR_ERR_INVALID_SCENE;
        if ((uint64_t)v->curve_vertex_pos[i] + (uint64_t)(t & 7) > v->n_vertices) return SPR_ERR_INVALID_SCENE;
        const uint32_t p = v->curve_path_id[i];
        if (p >= v->n_paths || p < last) return SPR_ERR_INVALID_SCENE;
        last = p;
    }
    for (uint32_t i = 0; i < v->n_vertices; ++i)
        if (v->vertex_path_id[i] >= v->n_paths) return SPR_ERR_INVALID_SCENE;
    return SPR_OK;
}

template <class T>
int upload(DevBuf &b, const T *src, size_t n) {
    int st = ensure(b, n * sizeof(T));
    if (st) return st;
    if (n && cudaMemcpy(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return cuda_status();
    return SPR_OK;
}

void rec(spr_handle *h, int i, cudaStream_t s) {
    if (h->timing) cudaEventRecord(h->ev[i], s);
}

}  // namespace

extern "C" {

int spr_create(const spr_config *config, spr_handle **out) {
    if (!config || !out) return SPR_ERR_INVALID_ARG;
    *out = nullptr;
    int st = validate_config(config);
    if (st) return st;
    if (cudaSetDevice(config->device) != cudaSuccess) return cuda_status();
    spr_handle *h = new (std::nothrow) spr_handle();
    if (!h) return SPR_ERR_OUT_OF_MEMORY;
    h->cfg = *config;
    for (DevBuf *b : handle_bufs(h)) b->budget = &h->budget;
    for (int i = 0; i < 16; ++i) h->m[i] = (i % 5 == 0) ? 1.f : 0.f;
    st = build_tables(h);
    if (!st) {
        ResolveTables rt;
        build_resolve_tables(&rt);
        st = upload(h->rtables, &rt, 1);
    }
    if (!st) st = ensure(h->counters, sizeof(FrameCounters));
    if (!st && cudaMallocHost((void **)&h->h_counters, sizeof(FrameCounters)) != cudaSuccess) st = cuda_status();
    if (!st && cudaMallocHost((void **)&h->h_u32, 64) != cudaSuccess) st = cuda_status();
    if (st) {
        spr_destroy(h);
        return st;
    }
    *out = h;
    return SPR_OK;
}

int spr_destroy(spr_handle *h) {
    if (!h) return SPR_OK;
    cudaSetDevice(h->cfg.device);
    drop_graph(h);
    if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
    if (h->done_ev) cudaEventDestroy(h->done_ev);
    for (DevBuf *b : handle_bufs(h)) b->release();
    if (h->h_counters) cudaFreeHost(h->h_counters);
    if (h->h_u32) cudaFreeHost(h->h_u32);
    for (auto &e : h->ev)
        if (e) cudaEventDestroy(e);
    delete h;
    return SPR_OK;
}

int spr_resize(spr_handle *h, int32_t width, int32_t height) {
    if (!h) return SPR_ERR_INVALID_ARG;
    drop_graph(h);
    h->caps_ok = false;
    spr_config c = h->cfg;
    c.width = width;
    c.height = height;
    int st = validate_config(&c);
    if (st) return st;
    h->cfg = c;
    h->frame_valid = false;
    return SPR_OK;
}

int spr_set_samples(spr_handle *h, int32_t samples) {
    if (!h) return SPR_ERR_INVALID_ARG;
    drop_graph(h);
    h->caps_ok = false;
    if (samples != 8 && samples != 16 && samples != 32 && samples != 256) return SPR_ERR_INVALID_ARG;
    if (samples == 256 && !h->cfg.ms_output) return SPR_ERR_INVALID_ARG;
    cudaSetDevice(h->cfg.device);
    h->cfg.samples = samples;
    h->frame_valid = false;
    return build_tables(h);
}

int spr_set_multisample_output(spr_handle *h, int32_t enable) {
    if (!h) return SPR_ERR_INVALID_ARG;
    drop_graph(h);
    if (!enable && h->cfg.samples == 256) return SPR_ERR_INVALID_ARG;
    h->cfg.ms_output = enable ? 1 : 0;
    return SPR_OK;
}

int spr_enable_srgb_correction(spr_handle *h, int32_t enable) {
    if (!h) return SPR_ERR_INVALID_ARG;
    drop_graph(h);
    h->cfg.srgb = enable ? 1 : 0;
    return SPR_OK;
}

}  // extern "C"

namespace {

// Host path of spr_set_scene (validation and orientation on the CPU), for
// scenes whose curves share or reorder vertex ranges.
int set_scene_host(spr_handle *h, const spr_scene_view *v) {
    int st = validate_scene(v);
    if (st) return st;
    const uint32_t P = v->n_paths, C = v->n_curves, V = v->n_vertices;
    // unifyCurveVertexOrder (ras_base.cpp:523-569): reverse a curve unless
    // (y_first, x_first) < (y_last, x_last) comparing float bit patterns.
    std::vector<float> vert(v->vertex, v->vertex + 2 * (size_t)V);
    std::vector<CurveDesc> cd(C);
    std::vector<uint32_t> vmap(V);
    for (uint32_t i = 0; i < V; ++i) vmap[i] = i;
    for (uint32_t i = 0; i < C; ++i) {
        const int type = v->curve_type[i];
        const int vn = type & 7;
        const uint32_t p = v->curve_vertex_pos[i];
        uint32_t bxf, byf, bxl, byl;
        std::memcpy(&bxf, &vert[2 * p], 4);
        std::memcpy(&byf, &vert[2 * p + 1], 4);
        std::memcpy(&bxl, &vert[2 * (p + vn - 1)], 4);
        std::memcpy(&byl, &vert[2 * (p + vn - 1) + 1], 4);
        uint32_t rev = 0;
        if (!(byf < byl || (byf == byl && bxf < bxl))) {
            rev = 1;
            for (int k = 0; k < vn; ++k) vmap[p + k] = p + vn - 1 - k;
            for (int k = 0; k < vn / 2; ++k) {
                std::swap(vert[2 * (p + k)], vert[2 * (p + vn - k - 1)]);
                std::swap(vert[2 * (p + k) + 1], vert[2 * (p + vn - k - 1) + 1]);
            }
        }
        cd[i].vpos = p;
        cd[i].pid = v->curve_path_id[i];
        cd[i].w = type == SPR_CURVE_RATIONAL ? v->curve_arc_w[i] : 0.f;
        cd[i].type = (uint32_t)type | (rev << 8);
    }
    if ((st = upload(h->vertex, vert.data(), vert.size()))) return st;
    if ((st = upload(h->vmap, vmap.data(), vmap.size()))) return st;
    if ((st = upload(h->vpid, v->vertex_path_id, V))) return st;
    if ((st = upload(h->curves, cd.data(), C))) return st;
    if ((st = upload(h->rule, v->path_fill_rule, P))) return st;
    if ((st = upload(h->fill, v->path_fill_rgba, P))) return st;
    h->has_affine = v->path_affine != nullptr;
    if (h->has_affine && (st = upload(h->affine, v->path_affine, 6 * (size_t)P))) return st;
    h->P = P;
    h->C = C;
    h->V = V;
    h->has_scene = true;
    return SPR_OK;
}

}  // namespace

extern "C" {

int spr_set_scene(spr_handle *h, const spr_scene_view *v) {
    if (!h) return SPR_ERR_INVALID_ARG;
    drop_graph(h);
    // the frame capacities stay when the new scene has the same element
    // counts (the same scene again, or new geometry of the same structure);
    // a frame that outgrows them is rendered again, sized, when read
    const bool keep_caps = h->caps_ok && h->has_scene && h->n_scenes == 0 && v != nullptr &&
                           v->n_paths == h->P && v->n_curves == h->C && v->n_vertices == h->V;
    h->caps_ok = false;
    int st = validate_view(v);
    if (st) return st;
    cudaSetDevice(h->cfg.device);
    h->has_scene = false;
    h->frame_valid = false;
    h->n_scenes = 0;
    const uint32_t P = v->n_paths, C = v->n_curves, V = v->n_vertices;
    // the caller's arrays straight to the device, then validation and
    // orientation there (one read-back of the flags)
    if ((st = ensure(h->vertex, 8 * (size_t)V)) || (st = ensure(h->vpid, 4 * (size_t)V)) ||
        (st = ensure(h->vmap, 4 * (size_t)V)) || (st = ensure(h->curves, sizeof(CurveDesc) * (size_t)C)) ||
        (st = ensure(h->sc_vpos, 4 * (size_t)C)) || (st = ensure(h->sc_type, (size_t)C)) ||
        (st = ensure(h->sc_pid, 4 * (size_t)C)) || (st = ensure(h->sc_w, 4 * (size_t)C)) ||
        (st = ensure(h->rule, (size_t)P)) || (st = ensure(h->fill, 4 * (size_t)P)) ||
        (st = ensure(h->scene_flags, 4)) || (v->path_affine && (st = ensure(h->affine, 24 * (size_t)P))))
        return st;
    cudaStream_t s = nullptr;
    auto put = [&](DevBuf &b, const void *src, size_t bytes) {
        if (bytes) cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, s);
    };
    put(h->vertex, v->vertex, 8 * (size_t)V);
    put(h->vpid, v->vertex_path_id, 4 * (size_t)V);
    put(h->sc_vpos, v->curve_vertex_pos, 4 * (size_t)C);
    put(h->sc_type, v->curve_type, (size_t)C);
    put(h->sc_pid, v->curve_path_id, 4 * (size_t)C);
    if (v->curve_arc_w) put(h->sc_w, v->curve_arc_w, 4 * (size_t)C);
    put(h->rule, v->path_fill_rule, (size_t)P);
    put(h->fill, v->path_fill_rgba, 4 * (size_t)P);
    if (v->path_affine) put(h->affine, v->path_affine, 24 * (size_t)P);
    cudaMemsetAsync(h->scene_flags.p, 0, 4, s);
    launch_scene_prepare(h->sc_vpos.as<uint32_t>(), h->sc_type.as<uint8_t>(), h->sc_pid.as<uint32_t>(),
                         v->curve_arc_w ? h->sc_w.as<float>() : nullptr, C, V, P, h->vertex.as<float2>(),
                         h->vpid.as<uint32_t>(), h->vmap.as<uint32_t>(), h->curves.as<CurveDesc>(),
                         h->scene_flags.as<uint32_t>(), s);
    cudaMemcpyAsync(h->h_u32, h->scene_flags.p, 4, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status();
    if ((st = cuda_status())) return st;
    const uint32_t flags = h->h_u32[0];
    if (flags & 1u) return SPR_ERR_INVALID_SCENE;
    h->scene_on_device = false;
    if (flags & 2u) return set_scene_host(h, v);
    h->scene_on_device = true;
    h->scene_has_arcw = v->curve_arc_w != nullptr;
    h->has_affine = v->path_affine != nullptr;
    h->P = P;
    h->C = C;
    h->V = V;
    h->has_scene = true;
    h->caps_ok = keep_caps;
    return SPR_OK;
}

int spr_validate_scene(const spr_scene_view *scene) { return validate_scene(scene); }

int spr_set_transform(spr_handle *h, const float m[16]) {
    if (!h || !m) return SPR_ERR_INVALID_ARG;
    drop_graph(h);
    std::memcpy(h->m, m, sizeof(h->m));
    return SPR_OK;
}

}  // extern "C"

namespace {

// A differentiable frame: the resolve step becomes the float composite
// (forward) or its adjoint (backward).  Pointers are device pointers.
struct DiffCall {
    bool backward;
    const float *fill;        // 4 per path
    const float *grad_image;  // 4 per pixel (backward)
    float *image;             // 4 per pixel (forward)
    float *grad_fill;         // 4 per path (backward)
    float *grad_vertex;       // 2 per input vertex (backward)
    float *grad_affine;       // 6 per path, or null (backward)
    // pass `pass` of `passes` (256-sample frames: 8 passes, each weighted
    // `scale`; the forward adds its image to the earlier passes', the
    // backward sums the passes' gradients and maps vertices after the last)
    int pass = 0, passes = 1;
    float scale = 1.f;
};

int diff_stage(spr_handle *h, const FrameArgs &a, const DiffCall &dc, const uint32_t *pv, const uint32_t *bstart,
               const uint32_t *bend, cudaStream_t s, int *L) {
    DiffArgs d{};
    d.fill = reinterpret_cast<const float4 *>(dc.fill);
    d.grad_image = reinterpret_cast<const float4 *>(dc.grad_image);
    d.image = reinterpret_cast<float4 *>(dc.image);
    d.grad_fill = reinterpret_cast<float4 *>(dc.grad_fill);
    d.draw = h->draw.as<int4>();
    d.merged = h->merged.as<uint32_t>();
    d.pval = pv;
    d.bstart = bstart;
    d.bend = bend;
    d.npairs = pv ? h->npairs : 0;
    if (d.npairs > 0) {
        int st = ensure(h->bitems, 48 * (size_t)d.npairs);
        if (st) return st;
        d.bitem = h->bitems.as<uint4>();
        d.bfill = reinterpret_cast<float4 *>(d.bitem + d.npairs);
        d.bmm = d.bitem + 2 * d.npairs;
    }
    d.chord = h->chord.as<float4>();
    d.lmask = h->lmask.as<uint32_t>();
    d.vmask = h->vmask.as<uint32_t>();
    d.pidw = h->pidw.as<uint32_t>();
    d.perm = h->perm_sorted;
    d.heads = h->heads.as<uint32_t>();
    d.item_path = h->item_path.as<uint32_t>();
    d.skey = h->skey_sorted;
    d.wn_scan = h->wn_scan.as<int8_t>();
    d.entries = h->entries.as<int2>();
    d.tvert = h->tvert.as<float2>();
    d.nf = h->nf;
    FrameCounters *ctr = h->counters.as<FrameCounters>();
    d.queue = &ctr->bin_queue;
    d.status = &ctr->diff_status;
    d.out_scale = dc.scale;
    d.accumulate = dc.pass > 0 ? 1 : 0;
    if (!dc.backward) {
        *L += launch_diff_forward(a, d, s);
        return cuda_status();
    }
    int st = ensure(h->grad_tvert, 8 * (size_t)std::max<uint32_t>(h->V, 1));
    if (st) return st;
    if ((st = ensure(h->chain, 16 * (size_t)std::max<int64_t>(h->nf, 1) + 16))) return st;
    d.grad_tvert = h->grad_tvert.as<float2>();
    const bool multi = dc.passes > 1;  // the pass's gradients go to staging buffers first
    if (multi) {
        if ((st = ensure(h->gfill_pass, 16 * (size_t)std::max<uint32_t>(h->P, 1))) ||
            (st = ensure(h->gtvert_total, 8 * (size_t)std::max<uint32_t>(h->V, 1))))
            return st;
        d.grad_fill = h->gfill_pass.as<float4>();
    }
    d.chain = h->chain.as<float4>() + 1;
    d.n_chain = reinterpret_cast<uint32_t *>(h->chain.p);
    for (int depth = h->tape_depth;; depth *= 2) {
        const int64_t words = diff_tape_words(a, depth);
        if ((st = ensure(h->tape, 16 * (size_t)words)) ||
            (st = ensure(h->tape_rec, 16 * (size_t)diff_tape_rec_words(a, depth))))
            return st;
        d.tape = h->tape.as<float4>();
        d.tape_rec = h->tape_rec.as<float4>();
        d.tape_depth = depth;
        cudaMemsetAsync(d.grad_fill, 0, 16 * (size_t)h->P, s);
        cudaMemsetAsync(h->grad_tvert.p, 0, 8 * (size_t)h->V, s);
        cudaMemsetAsync(&ctr->diff_status, 0, 4, s);
        cudaMemsetAsync(d.n_chain, 0, 4, s);
        *L += launch_diff_backward(a, d, s);
        cudaMemcpyAsync(h->h_u32, &ctr->diff_status, 4, cudaMemcpyDeviceToHost, s);
        ++h->host_syncs;
        if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status();
        if (!(h->h_u32[0] & 1u)) {
            h->tape_depth = depth;
            break;
        }
        if (depth >= (1 << 16)) return SPR_ERR_CAPACITY_EXCEEDED;
    }
    const float2 *gt = h->grad_tvert.as<float2>();
    if (multi) {
        *L += launch_accumulate(dc.grad_fill, reinterpret_cast<float *>(d.grad_fill), 4 * (int64_t)h->P, dc.pass == 0,
                                s);
        *L += launch_accumulate(h->gtvert_total.as<float>(), h->grad_tvert.as<float>(), 2 * (int64_t)h->V,
                                dc.pass == 0, s);
        if (dc.pass + 1 < dc.passes) return cuda_status();
        gt = h->gtvert_total.as<float2>();
    }
    if (dc.grad_affine) cudaMemsetAsync(dc.grad_affine, 0, 24 * (size_t)h->P, s);
    *L += launch_diff_vertex(a, gt, h->vmap.as<uint32_t>(),
                             reinterpret_cast<float2 *>(dc.grad_vertex), dc.grad_affine, s);
    return cuda_status();
}

// Words of the bin arrays: offsets (n_bins + 1), counts, fill counters, each
// padded to 16 bytes.
int64_t bin_stride(int64_t nbins) { return (nbins + 1 + 3) & ~int64_t(3); }
int64_t bin_words(int64_t nbins) { return 3 * bin_stride(nbins); }

// The batch scene table for bin geometry `shift` (tiles of 1 << shift
// columns): every scene's tile and band counts and first bin, uploaded when
// the geometry differs from the table's.
int scene_bins(spr_handle *h, int shift, cudaStream_t s) {
    if (h->n_scenes == 0 || h->scenes_shift == shift) return SPR_OK;
    uint64_t bins = 0;
    for (SceneInfo &si : h->scenes_h) {
        si.ntx = bin_cols(si.W, shift);
        si.nrows = bin_rows(si.H, shift);
        si.bin_off = (uint32_t)bins;
        bins += (uint64_t)si.ntx * (uint64_t)si.nrows;
        if (bins > UINT32_MAX) return SPR_ERR_CAPACITY_EXCEEDED;
    }
    // (from pageable memory: staged before the call returns)
    if (cudaMemcpyAsync(h->scenes_d.p, h->scenes_h.data(), sizeof(SceneInfo) * h->scenes_h.size(),
                        cudaMemcpyHostToDevice, s) != cudaSuccess)
        return cuda_status();
    h->scenes_shift = shift;
    return SPR_OK;
}

// Headroom of the capacities a sized frame sets, so that frames whose sizes
// drift a little (an animation, a fitting loop) keep fitting.
int64_t with_headroom(int64_t n) { return n + n / 8 + 256; }

// The counters of a frame rendered without host reads, once complete:
// sizes to the host, or the frame rendered again (sized) if it outgrew its
// buffers.  Every call that reads a frame's results settles it first.
int render_frame(spr_handle *h, void *stream, const DiffCall *dc);

// Queues the copy of a frame's counters to the host and the event after it
// (a frame rendered without host reads).
int mark_pending(spr_handle *h, cudaStream_t s) {
    if (!h->done_ev && cudaEventCreateWithFlags(&h->done_ev, cudaEventDisableTiming) != cudaSuccess)
        return cuda_status();
    cudaMemcpyAsync(h->h_counters, h->counters.p, sizeof(FrameCounters), cudaMemcpyDeviceToHost, s);
    cudaEventRecord(h->done_ev, s);
    h->pending = true;
    h->pending_stale = false;
    h->pending_stream = s;
    return SPR_OK;
}

int settle(spr_handle *h) {
    if (!h->pending) return SPR_OK;
    h->pending = false;
    if (cudaEventSynchronize(h->done_ev) != cudaSuccess) return cuda_status();
    const FrameCounters c = *h->h_counters;
    if (c.status & kStatusTimeout) {
        h->frame_valid = false;
        return SPR_ERR_TIMEOUT;
    }
    if (c.status & kStatusOverflow) {
        h->caps_ok = false;
        if (h->pending_stale) {  // its inputs are gone: it cannot be rendered again
            h->frame_valid = false;
            return SPR_ERR_CAPACITY_EXCEEDED;
        }
        return render_frame(h, h->pending_stream, nullptr);
    }
    h->nf = c.nf;
    h->nm = c.n_merged;
    h->ns = c.n_span;
    h->npairs = c.n_pairs;
    h->en.curve_fragment = (int32_t)c.nf;
    h->en.merged_fragment = (int32_t)c.n_merged;
    h->en.span = (int32_t)c.n_span;
    return SPR_OK;
}

// A pending frame that a new frame supersedes: its overflow, if it is known
// already, still teaches the capacities (no waiting).
void supersede(spr_handle *h) {
    if (!h->pending) return;
    h->pending = false;
    if (cudaEventQuery(h->done_ev) == cudaSuccess && (h->h_counters->status & kStatusOverflow)) h->caps_ok = false;
    cudaGetLastError();  // (cudaErrorNotReady)
}

// Fragment sort choice: one block per path needs enough paths to fill the
// GPU and segments short enough for shared memory (longer ones are sorted by
// a single block, chunk by chunk).
constexpr int64_t kSegmentSortMinPaths = 1024;
constexpr int64_t kSegmentSortMaxMean = 2048;  // mean entries per path

// One frame.  Sized (differentiable frames, and the first frame after a
// change of scene, viewport or sample count): the entry count and then the
// pair count are read back as they are known, and the buffers and their
// capacities set from them.  Otherwise no host reads: every kernel takes
// its size from the device counters and its grid from the capacities, and
// the counters are copied to the host for settle().
int render_frame(spr_handle *h, void *stream, const DiffCall *dc) {
    if (!h) return SPR_ERR_INVALID_ARG;
    if (!h->has_scene) return SPR_ERR_NO_SCENE;
    cudaSetDevice(h->cfg.device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int st = build_tables(h);
    if (st) return st;
    supersede(h);
    h->frame_valid = false;
    h->diff_ready = false;
    int L = 0;  // kernels launched by this frame
    h->host_syncs = 0;
    if ((st = scene_bins(h, frame_bin_shift(h, dc != nullptr), s))) return st;
    FrameArgs a = make_args(h, dc != nullptr);
    const int W = a.W, H = a.H, WORDS = a.S / 8;
    const bool batch = h->n_scenes > 0;
    const int64_t npix = frame_pixels(h);
    // (the passes of a 256-sample frame are sized: they add up into one image)
    const bool sized = (dc != nullptr || !h->caps_ok || h->cfg.samples == 256) && !h->capturing;
    if (!sized) a.alt_shift = -1;  // (only a sized frame chooses the built-in tile)
    if (h->timing) {
        for (auto &e : h->ev)
            if (!e) cudaEventCreate(&e);
    }
    FrameCounters *ctr = h->counters.as<FrameCounters>();
    int64_t nbins = a.n_bins;
    // stage 3: transform + visibility
    if ((st = ensure(h->tvert, sizeof(float2) * h->V)) || (st = ensure(h->pflags, 4 * (size_t)h->P)) ||
        (st = ensure(h->pvis, h->P)) || (st = ensure(h->counts, 4 * (size_t)h->C + 16)) ||
        (st = ensure(h->offsets, 4 * ((size_t)h->C + 1) + 16)) ||
        (st = ensure(h->lb_off, 8 * (size_t)lookback_words(h->C))) || (st = ensure(h->image, 4 * (size_t)npix)) ||
        (st = ensure(h->bins, 4 * (size_t)bin_words(nbins))) ||
        (st = ensure(h->lb_pair, 8 * (size_t)lookback_words(nbins))) ||
        (st = ensure(h->overflow, 4 * (size_t)std::max<int64_t>(resolve_overflow_words(a), 1))))
        return st;
    cudaMemsetAsync(h->counters.p, 0, sizeof(FrameCounters), s);
    rec(h, 0, s);
    L += launch_transform(a, h->tvert.as<float2>(), h->pflags.as<uint32_t>(), h->pvis.as<uint8_t>(), s);
    rec(h, 1, s);
    // stages 4-5: monotone pieces, entry counts, offsets (single-pass scan)
    L += launch_curve_count(a, h->tvert.as<float2>(), h->pvis.as<uint8_t>(), h->counts.as<uint32_t>(), s);
    cudaMemsetAsync(h->lb_off.p, 0, 8 * (size_t)lookback_words(h->C), s);
    L += scan_lookback_u32(h->counts.as<uint32_t>(), h->offsets.as<uint32_t>(), nullptr, h->C, h->lb_off.as<uint64_t>(),
                           &ctr->tiles[0], h->lb_spin_cap, &ctr->status, &ctr->need_nf, s, h->lb_hold_tile);
    if (sized) {
        cudaMemcpyAsync(h->h_u32, &ctr->need_nf, 4, cudaMemcpyDeviceToHost, s);
        ++h->host_syncs;
        if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status();
        if ((st = cuda_status())) return st;
        const int64_t need = h->h_u32[0];
        if (need > INT32_MAX) return SPR_ERR_CAPACITY_EXCEEDED;
        h->cap_nf = dc ? std::max<int64_t>(need, 1) : with_headroom(need);
        h->cap_items = 2 * h->cap_nf;
    }
    const int64_t cap_nf = h->cap_nf, cap_items = h->cap_items;
    // stages 6-7: entries, fragments, boundary masks
    if ((st = ensure(h->entries, 8 * (size_t)cap_nf)) || (st = ensure(h->key, 4 * (size_t)cap_nf)) ||
        (st = ensure(h->pidw, 4 * (size_t)cap_nf)) || (st = ensure(h->wn, (size_t)cap_nf)) ||
        (st = ensure(h->mask, 4 * (size_t)WORDS * cap_nf)) ||
        // (16 entries past cap_nf of the sorted keys and positions: the
        // merged-mask pass copies whole 16-entry blocks)
        (st = ensure(h->skey[0], 8 * (size_t)cap_nf + 128)) || (st = ensure(h->skey[1], 8 * (size_t)cap_nf + 128)) ||
        (st = ensure(h->sval[0], 4 * (size_t)cap_nf + 64)) || (st = ensure(h->sval[1], 4 * (size_t)cap_nf + 64)) ||
        (st = ensure(h->wn_scan, (size_t)cap_nf)) ||
        (st = ensure(h->draw, 16 * (size_t)cap_items)) || (st = ensure(h->heads, 4 * (size_t)cap_nf)) ||
        (st = ensure(h->lb_mark, 8 * (size_t)scan_mark_status_words(cap_nf))) ||
        (st = ensure(h->merged, 4 * (size_t)WORDS * cap_nf)) ||
        (batch && (st = ensure(h->item_scene, 4 * (size_t)cap_items))))
        return st;
    uint32_t *item_scene = batch ? h->item_scene.as<uint32_t>() : nullptr;
    if (dc) {
        if ((st = ensure(h->chord, 16 * (size_t)cap_nf)) || (st = ensure(h->lmask, 4 * (size_t)WORDS * cap_nf)) ||
            (st = ensure(h->vmask, 4 * (size_t)WORDS * cap_nf)) || (st = ensure(h->item_path, 4 * (size_t)cap_items)))
            return st;
        a.chord = h->chord.as<float4>();
        a.lmask = h->lmask.as<uint32_t>();
        a.vmask = h->vmask.as<uint32_t>();
        a.item_path = h->item_path.as<uint32_t>();
    }
    L += launch_admit(&ctr->need_nf, &ctr->nf, (uint32_t)std::min<int64_t>(cap_nf, INT32_MAX), &ctr->status, s);
    rec(h, 2, s);
    // emission order: curves sorted by estimated cost (16-bit keys, two passes)
    const uint32_t *order = nullptr;
    if (h->tune_emit >= 0 ? h->tune_emit == 1 : h->C >= 4096) {
        if ((st = ensure(h->ekey[0], 4 * (size_t)h->C)) || (st = ensure(h->ekey[1], 4 * (size_t)h->C)) ||
            (st = ensure(h->eval[0], 4 * (size_t)h->C)) || (st = ensure(h->eval[1], 4 * (size_t)h->C)) ||
            (st = ensure(h->sort_tmp, 4 * (size_t)radix_tmp_words(std::max<int64_t>(cap_nf, h->C)))))
            return st;
        L += launch_emit_keys(a, h->counts.as<uint32_t>(), h->ekey[0].as<uint32_t>(), h->eval[0].as<uint32_t>(), s);
        int el = 0;
        const bool ealt = radix_sort<uint32_t>(h->ekey[0].as<uint32_t>(), h->eval[0].as<uint32_t>(),
                                               h->ekey[1].as<uint32_t>(), h->eval[1].as<uint32_t>(), h->C, 16,
                                               h->sort_tmp.as<uint32_t>(), s, &el);
        L += el;
        order = ealt ? h->eval[1].as<uint32_t>() : h->eval[0].as<uint32_t>();
    }
    L += launch_curve_emit(a, h->tvert.as<float2>(), h->pvis.as<uint8_t>(), h->offsets.as<uint32_t>(), order,
                           h->entries.as<int2>(), ctr, s);
    L += launch_fragment(a, h->tvert.as<float2>(), h->entries.as<int2>(), cap_nf, ctr, h->key.as<int32_t>(),
                         h->pidw.as<uint32_t>(), h->wn.as<int8_t>(), h->mask.as<uint32_t>(),
                         h->skey[0].as<uint64_t>(), h->sval[0].as<uint32_t>(), s);
    rec(h, 3, s);
    // stage 8: stable sort by (path, cell key).  The entries arrive grouped by
    // path, so with enough paths to fill the GPU each path's segment is
    // sorted on its own by one block; frames of few (hence long) paths take
    // the device-wide LSD radix sort, whose work does not depend on them.
    int rl = 0;
    const bool segment_sort = h->tune_sort >= 0 ? h->tune_sort == 1
                                                : h->P >= kSegmentSortMinPaths &&
                                                      cap_nf / std::max<int64_t>(h->P, 1) <= kSegmentSortMaxMean;
    if (segment_sort && h->P > 0) {
        if ((st = ensure(h->path_start, 4 * ((size_t)h->P + 1)))) return st;
        L += launch_segment_sort(h->curves.as<CurveDesc>(), h->C, h->P, h->offsets.as<uint32_t>(),
                                 h->skey[0].as<uint64_t>(), h->sval[0].as<uint32_t>(), h->skey[1].as<uint64_t>(),
                                 h->sval[1].as<uint32_t>(), h->path_start.as<uint32_t>(), ctr, s);
        h->skey_sorted = h->skey[1].as<uint64_t>();
        h->perm_sorted = h->sval[1].as<uint32_t>();
    } else {
        if ((st = ensure(h->sort_tmp, 4 * (size_t)radix_tmp_words(std::max<int64_t>(cap_nf, h->C))))) return st;
        const int key_bits = 24 + bits_for(h->P ? h->P - 1 : 0);
        const bool alt = radix_sort<uint64_t>(h->skey[0].as<uint64_t>(), h->sval[0].as<uint32_t>(),
                                              h->skey[1].as<uint64_t>(), h->sval[1].as<uint32_t>(), cap_nf, key_bits,
                                              h->sort_tmp.as<uint32_t>(), s, &rl, &ctr->nf);
        L += rl;
        h->skey_sorted = alt ? h->skey[1].as<uint64_t>() : h->skey[0].as<uint64_t>();
        h->perm_sorted = alt ? h->sval[1].as<uint32_t>() : h->sval[0].as<uint32_t>();
    }
    rec(h, 4, s);
    // stages 9-12, 14: winding scan, marks, draw list (one look-back pass),
    // with the pairs of each resolve bin counted
    uint32_t *bin_off = h->bins.as<uint32_t>(), *bin_count = bin_off + bin_stride(nbins),
             *bin_fill = bin_count + bin_stride(nbins);
    cudaMemsetAsync(bin_count, 0, 8 * (size_t)bin_stride(nbins), s);
    cudaMemsetAsync(h->lb_mark.p, 0, 8 * (size_t)scan_mark_status_words(cap_nf), s);
    L += launch_scan_mark(a, cap_nf, h->skey_sorted, h->wn_scan.as<int8_t>(),
                          h->draw.as<int4>(), h->heads.as<uint32_t>(), item_scene, bin_count, ctr,
                          h->lb_mark.as<uint64_t>(),
                          h->lb_spin_cap, s);
    rec(h, 5, s);
    // stage 13: merged sample masks
    L += launch_stencil(a, cap_nf, ctr, h->skey_sorted, h->perm_sorted, h->mask.as<uint32_t>(),
                        h->wn_scan.as<int8_t>(), h->heads.as<uint32_t>(), h->merged.as<uint32_t>(), h->lb_spin_cap,
                        s);
    rec(h, 6, s);
    // stage 15: draw items binned by resolve tile (a band of cell rows x columns): bin offsets
    // from the counts, then the items placed and sorted per bin; resolve
    cudaMemsetAsync(h->lb_pair.p, 0, 8 * (size_t)lookback_words(nbins), s);
    L += scan_lookback_u32(bin_count, bin_off, nullptr, nbins, h->lb_pair.as<uint64_t>(), &ctr->tiles[2],
                           h->lb_spin_cap, &ctr->status, &ctr->need_pairs, s);
    if (sized) {
        cudaMemcpyAsync(h->h_counters, h->counters.p, sizeof(FrameCounters), cudaMemcpyDeviceToHost, s);
        ++h->host_syncs;
        if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status();
        if ((st = cuda_status())) return st;
        if (h->h_counters->status & kStatusTimeout) return SPR_ERR_TIMEOUT;
        h->nf = h->h_counters->nf;
        h->nm = h->h_counters->n_merged;
        h->ns = h->h_counters->n_span;
        h->npairs = h->h_counters->need_pairs;
        h->cap_pairs = dc ? std::max<int64_t>(h->npairs, 1) : with_headroom(h->npairs);
        if (!dc) {  // the built-in tile, from this frame's spans
            const uint64_t items = (uint64_t)h->h_counters->n_merged + h->h_counters->n_span;
            h->auto_bin_shift = h->h_counters->span_px <= (uint64_t)kShortSpanPx * items ? kPlainBinShift : kBinShift;
            if (frame_bin_shift(h, false) != a.bin_shift) {
                // the bins again in that tile: counts from the draw list, offsets, pair total
                if ((st = scene_bins(h, frame_bin_shift(h, false), s))) return st;
                a = make_args(h, false);
                nbins = a.n_bins;
                if ((st = ensure(h->bins, 4 * (size_t)bin_words(nbins))) ||
                    (st = ensure(h->lb_pair, 8 * (size_t)lookback_words(nbins))))
                    return st;
                bin_off = h->bins.as<uint32_t>();
                bin_count = bin_off + bin_stride(nbins);
                bin_fill = bin_count + bin_stride(nbins);
                cudaMemsetAsync(bin_count, 0, 8 * (size_t)bin_stride(nbins), s);
                L += launch_bin_count(a, h->draw.as<int4>(), item_scene, cap_items, ctr, bin_count, s);
                cudaMemsetAsync(h->lb_pair.p, 0, 8 * (size_t)lookback_words(nbins), s);
                cudaMemsetAsync(&ctr->tiles[2], 0, 4, s);
                L += scan_lookback_u32(bin_count, bin_off, nullptr, nbins, h->lb_pair.as<uint64_t>(), &ctr->tiles[2],
                                       h->lb_spin_cap, &ctr->status, &ctr->need_pairs, s);
                h->npairs = h->h_counters->pairs_alt;  // (the total the scan-mark pass counted for this tile)
                h->cap_pairs = with_headroom(h->npairs);
            }
        }
    }
    const int64_t cap_pairs = h->cap_pairs;
    if ((st = ensure(h->pval, 4 * (size_t)cap_pairs))) return st;
    // resolve records of plain frames (the adjoint reads the items and masks itself)
    if (!dc && ((st = ensure(h->rec_a, 8 * (size_t)cap_pairs)) ||
                (st = ensure(h->rec_m, 4 * (size_t)WORDS * cap_pairs))))
        return st;
    L += launch_admit(&ctr->need_pairs, &ctr->n_pairs, (uint32_t)std::min<int64_t>(cap_pairs, INT32_MAX),
                      &ctr->status, s);
    L += launch_bin_scatter(a, h->draw.as<int4>(), item_scene, cap_items, ctr, bin_off, bin_fill,
                            h->pval.as<uint32_t>(), s);
    L += launch_bin_sort(bin_off, nbins, h->pval.as<uint32_t>(), ctr, a.S, a.bin_shift, h->draw.as<int4>(),
                         h->merged.as<uint32_t>(), dc ? nullptr : h->rec_a.as<uint2>(),
                         dc ? nullptr : h->rec_m.as<uint32_t>(), s);
    const uint32_t *pv = h->pval.as<uint32_t>();
    uint32_t *bin_start = bin_off, *bin_end = bin_off + 1;
    rec(h, 7, s);
    h->en.path = (int32_t)h->P;
    h->en.curve = (int32_t)h->C;
    h->en.vertex = (int32_t)h->V;
    if (sized) {
        h->en.curve_fragment = (int32_t)h->nf;
        h->en.merged_fragment = (int32_t)h->nm;
        h->en.span = (int32_t)h->ns;
    }
    if (dc) {
        if ((st = diff_stage(h, a, *dc, pv, bin_start, bin_end, s, &L))) return st;
    } else {
        L += launch_resolve(a, h->rec_a.as<uint2>(), h->rec_m.as<uint32_t>(), bin_start, bin_end,
                            h->image.as<uint32_t>(), h->overflow.as<uint32_t>(), ctr, s);
    }
    rec(h, 8, s);
    if ((st = cuda_status())) return st;
    if (h->timing) {
        cudaEventSynchronize(h->ev[8]);
        for (int i = 0; i < kSteps; ++i) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, h->ev[i], h->ev[i + 1]);
            h->step_ms[i] = ms;
        }
    }
    if (sized) {
        h->caps_ok = true;
    } else if (!h->capturing) {
        if ((st = mark_pending(h, s))) return st;  // the counters come back on their own; settle() reads them
    }
    h->launches = L;
    h->pv_sorted = pv;
    h->diff_ready = dc && !dc->backward;
    h->frame_valid = true;
    h->frame_W = W;
    h->frame_H = H;
    h->frame_S = a.S;
    return cuda_status();
}

// Backward of the differentiable forward frame still held in the buffers
// (nothing changed since): the adjoint kernels only.
int backward_of_held_frame(spr_handle *h, void *stream, const DiffCall &dc) {
    cudaSetDevice(h->cfg.device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (int st = scene_bins(h, kBinShift, s)) return st;
    FrameArgs a = make_args(h, true);
    if (h->nf > 0) {
        a.chord = h->chord.as<float4>();
        a.lmask = h->lmask.as<uint32_t>();
        a.vmask = h->vmask.as<uint32_t>();
        a.item_path = h->item_path.as<uint32_t>();
    }
    int L = 0;
    h->host_syncs = 0;
    uint32_t *bin_start = h->bins.as<uint32_t>();  // (bin b's items end where bin b + 1's start)
    const int st = diff_stage(h, a, dc, h->pv_sorted, bin_start, bin_start + 1, s, &L);
    h->launches = L;
    return st ? st : cuda_status();
}

// A 256-sample frame: 8 passes of 32 samples (pass g: rows 8j + g of the
// 256-row pattern, geometry moved by -pass_shift_256(g)), each a whole
// frame.  Plain frames add the passes' exact fixed-point sample sums and
// encode once; differentiable frames add the passes' images and gradients
// with weight 1/8.  Launch, host-read and step-time figures are the passes'
// totals; the element counts and stage dumps are the last pass's.
int render_passes(spr_handle *h, void *stream, const DiffCall *dc) {
    if (!h->has_scene) return SPR_ERR_NO_SCENE;
    cudaSetDevice(h->cfg.device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t npix = frame_pixels(h);
    int st = SPR_OK;
    if (!dc) {
        if ((st = ensure(h->sums, 32 * (size_t)npix))) return st;
        cudaMemsetAsync(h->sums.p, 0, 32 * (size_t)npix, s);
    }
    int launches = 0, syncs = 0;
    double ms[kSteps] = {};
    for (int g = 0; g < kPasses256 && !st; ++g) {
        h->pass = g;
        if (dc) {
            DiffCall pc = *dc;
            pc.pass = g;
            pc.passes = kPasses256;
            pc.scale = 1.f / (float)kPasses256;
            st = render_frame(h, stream, &pc);
        } else {
            st = render_frame(h, stream, nullptr);
        }
        launches += h->launches;
        syncs += h->host_syncs;
        for (int i = 0; i < kSteps; ++i) ms[i] += h->step_ms[i];
    }
    h->pass = 0;
    h->diff_ready = false;  // the buffers hold the last pass only
    if (st) {
        h->frame_valid = false;
        return st;
    }
    if (!dc) launches += launch_encode_sums(make_args(h), h->sums.as<long long>(), h->image.as<uint32_t>(), npix, s);
    h->launches = launches;
    h->host_syncs = syncs;
    if (h->timing) std::memcpy(h->step_ms, ms, sizeof(ms));
    return cuda_status();
}

// One frame of any sample count.
int frame(spr_handle *h, void *stream, const DiffCall *dc) {
    if (h->cfg.samples == 256) return render_passes(h, stream, dc);
    return render_frame(h, stream, dc);
}

// A backward: after a differentiable forward of the same inputs (and with
// step timing off) the held frame's buffers are reused, else every stage is
// recomputed.
int backward_frame(spr_handle *h, void *stream, const DiffCall &dc) {
    if (h->diff_ready && !h->timing) return backward_of_held_frame(h, stream, dc);
    return frame(h, stream, &dc);
}

}  // namespace

extern "C" {

int spr_render(spr_handle *h, void *stream) {
    if (!h) return SPR_ERR_INVALID_ARG;
    if (!h->graph_mode || h->timing || !h->has_scene || h->cfg.samples == 256) return frame(h, stream, nullptr);
    cudaSetDevice(h->cfg.device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (h->gexec && (h->gexec_gen != g_alloc_gen.load() || !h->caps_ok)) drop_graph(h, false);  // buffers moved
    int st0 = SPR_OK;
    if (h->gexec) {
        supersede(h);
        if (cudaGraphLaunch(h->gexec, s) != cudaSuccess) return cuda_status();
        if ((st0 = mark_pending(h, s))) return st0;
        h->host_syncs = 0;
        h->frame_valid = true;
        ++h->graph_replays;
        return cuda_status();
    }
    // render this frame (sized if the capacities are not known), then
    // capture the launch sequence of a frame without host reads: it depends
    // on the capacities only, so replays stay valid while the sizes fit
    int st = render_frame(h, stream, nullptr);
    if (st || h->graph_failed) return st;
    if ((st = settle(h))) return st;
    if (!h->cap_stream && cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking) != cudaSuccess)
        return cuda_status();
    const uint64_t gen = g_alloc_gen.load();
    const int host_syncs = h->host_syncs, launches = h->launches;
    const spr_element_number en = h->en;
    const int64_t nf = h->nf, nm = h->nm, ns = h->ns, npairs = h->npairs;
    cudaGraph_t g = nullptr;
    bool ok = cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeRelaxed) == cudaSuccess;
    if (ok) {
        h->capturing = true;
        const int cst = render_frame(h, h->cap_stream, nullptr);
        h->capturing = false;
        ok = cudaStreamEndCapture(h->cap_stream, &g) == cudaSuccess && cst == SPR_OK && g != nullptr;
    }
    ok = ok && g_alloc_gen.load() == gen && cudaGraphInstantiate(&h->gexec, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (!ok) {  // stay eager for this scene
        cudaGetLastError();
        if (h->gexec) cudaGraphExecDestroy(h->gexec);
        h->gexec = nullptr;
        h->graph_failed = true;
    }
    h->gexec_gen = gen;
    h->host_syncs = host_syncs;
    h->launches = launches;
    h->en = en;
    h->nf = nf, h->nm = nm, h->ns = ns, h->npairs = npairs;
    h->frame_valid = true;
    return SPR_OK;
}

int spr_set_gradients(spr_handle *h, const uint32_t *table, uint32_t n_entries, const uint32_t *ramp,
                      uint32_t n_texels) {
    if (!h) return SPR_ERR_INVALID_ARG;
    drop_graph(h);
    if (!table || n_entries == 0) {
        h->n_grad = 0;
        return SPR_OK;
    }
    const int chk = check_gradients(table, n_entries, ramp, n_texels);
    if (chk) return chk;
    cudaSetDevice(h->cfg.device);
    int st = upload(h->grad_table, table, (size_t)12 * n_entries);
    if (!st) st = upload(h->grad_ramp, ramp, n_texels);
    if (st) return st;
    h->n_grad = n_entries;
    return SPR_OK;
}

int spr_set_rev_transform(spr_handle *h, const float ctx[13]) {
    if (!h || !ctx) return SPR_ERR_INVALID_ARG;
    drop_graph(h);
    std::memcpy(h->rev, ctx, sizeof(h->rev));
    return SPR_OK;
}

namespace {
// Mean device time of `frames` frames (after one untimed frame).
int time_frames(spr_handle *h, void *stream, int frames, float *ms) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int st = frame(h, stream, nullptr);
    if (st) return st;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return cuda_status();
    cudaEventRecord(e0, s);
    for (int i = 0; i < frames && !st; ++i) st = frame(h, stream, nullptr);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / (float)frames;
    return st ? st : cuda_status();
}
}  // namespace

int spr_autotune(spr_handle *h, int32_t frames, void *stream, spr_tune *out) {
    if (!h || frames < 1) return SPR_ERR_INVALID_ARG;
    if (!h->has_scene) return SPR_ERR_NO_SCENE;
    cudaSetDevice(h->cfg.device);
    drop_graph(h, false);
    const bool timing = h->timing;
    h->timing = false;
    h->tune_sort = h->tune_emit = -1;
    h->tune_bps = 0;
    const int bin_w0 = h->tune_bin_w;
    h->tune_bin_w = 0;
    if (bin_w0 != 0) h->caps_ok = false;  // (the pairs depend on the tile)
    float base = 0.f;
    int st = time_frames(h, stream, frames, &base);
    // one choice at a time, the others at their best so far
    int best_sort = -1, best_emit = -1, best_bps = 0;
    float best = base;
    for (int v = 0; v <= 1 && !st; ++v) {
        h->tune_sort = v;
        float t = 0.f;
        if ((st = time_frames(h, stream, frames, &t))) break;
        if (t < best) best = t, best_sort = v;
    }
    h->tune_sort = best_sort;
    for (int v = 0; v <= 1 && !st; ++v) {
        h->tune_emit = v;
        float t = 0.f;
        if ((st = time_frames(h, stream, frames, &t))) break;
        if (t < best) best = t, best_emit = v;
    }
    h->tune_emit = best_emit;
    for (int v = 2; v <= 3 && !st; ++v) {  // 4 is the default
        h->tune_bps = v;
        float t = 0.f;
        if ((st = time_frames(h, stream, frames, &t))) break;
        if (t < best) best = t, best_bps = v;
    }
    h->tune_bps = best_bps;
    int best_bin_w = 0;
    for (const int v : {64, 32, 16, 8}) {
        if (st) break;
        h->tune_bin_w = v;
        h->caps_ok = false;
        float t = 0.f;
        if ((st = time_frames(h, stream, frames, &t))) break;
        if (t < best) best = t, best_bin_w = v;
    }
    if (h->tune_bin_w != best_bin_w) h->caps_ok = false;
    h->tune_bin_w = best_bin_w;
    h->timing = timing;
    if (st) return st;
    if (out) {
        out->sort = best_sort;
        out->emit_order = best_emit;
        out->resolve_bps = best_bps;
        out->bin_width = best_bin_w;
        out->frame_ms = best;
        out->default_ms = base;
    }
    return SPR_OK;
}

int spr_set_tuning(spr_handle *h, const spr_tune *t) {
    if (!h || !t) return SPR_ERR_INVALID_ARG;
    if (t->sort < -1 || t->sort > 1 || t->emit_order < -1 || t->emit_order > 1 || t->resolve_bps < 0 ||
        t->resolve_bps > 4 ||
        (t->bin_width != 0 && t->bin_width != 64 && t->bin_width != 32 && t->bin_width != 16 && t->bin_width != 8))
        return SPR_ERR_INVALID_ARG;
    drop_graph(h, false);
    h->tune_sort = t->sort;
    h->tune_emit = t->emit_order;
    h->tune_bps = t->resolve_bps;
    const int bw = t->bin_width;  // (0: the built-in rule)
    if (bw != h->tune_bin_w) h->caps_ok = false;  // (the pairs depend on the tile)
    h->tune_bin_w = bw;
    return SPR_OK;
}

int spr_set_graph_replay(spr_handle *h, int32_t enable) {
    if (!h) return SPR_ERR_INVALID_ARG;
    h->graph_mode = enable != 0;
    if (!h->graph_mode) drop_graph(h, false);
    return SPR_OK;
}

int spr_graph_replays(spr_handle *h, int32_t *out) {
    if (!h || !out) return SPR_ERR_INVALID_ARG;
    *out = h->graph_replays;
    return SPR_OK;
}

int spr_update_vertices(spr_handle *h, const float *vertex, void *stream) {
    if (!h || !vertex) return SPR_ERR_INVALID_ARG;
    if (!h->has_scene) return SPR_ERR_NO_SCENE;
    if (!h->scene_on_device) return SPR_ERR_UNSUPPORTED;
    cudaSetDevice(h->cfg.device);
    // a captured frame reads the vertices from device memory and takes its
    // sizes from the device counters, so it stays valid for the moved
    // geometry: only the held differentiable frame and a pending frame's
    // inputs are gone
    h->diff_ready = false;
    if (h->pending) h->pending_stale = true;
    h->frame_valid = false;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (h->V && cudaMemcpyAsync(h->vertex.p, vertex, 8 * (size_t)h->V, cudaMemcpyDefault, s) != cudaSuccess)
        return cuda_status();
    cudaMemsetAsync(h->scene_flags.p, 0, 4, s);
    launch_scene_prepare(h->sc_vpos.as<uint32_t>(), h->sc_type.as<uint8_t>(), h->sc_pid.as<uint32_t>(),
                         h->scene_has_arcw ? h->sc_w.as<float>() : nullptr, h->C, h->V, h->P, h->vertex.as<float2>(),
                         h->vpid.as<uint32_t>(), h->vmap.as<uint32_t>(), h->curves.as<CurveDesc>(),
                         h->scene_flags.as<uint32_t>(), s);
    return cuda_status();
}

int spr_diff_render(spr_handle *h, const float *fill_rgba, float *image, void *stream) {
    if (!h || !fill_rgba || !image) return SPR_ERR_INVALID_ARG;
    if (h->n_scenes > 0) return SPR_ERR_UNSUPPORTED;
    const DiffCall dc{false, fill_rgba, nullptr, image, nullptr, nullptr, nullptr};
    return frame(h, stream, &dc);
}

int spr_diff_backward(spr_handle *h, const float *fill_rgba, const float *grad_image, float *grad_fill,
                      float *grad_vertex, float *grad_affine, void *stream) {
    if (!h || !fill_rgba || !grad_image || !grad_fill || !grad_vertex) return SPR_ERR_INVALID_ARG;
    if (h->n_scenes > 0) return SPR_ERR_UNSUPPORTED;
    if (grad_affine && !h->has_affine) return SPR_ERR_INVALID_ARG;
    const DiffCall dc{true, fill_rgba, grad_image, nullptr, grad_fill, grad_vertex, grad_affine};
    return backward_frame(h, stream, dc);
}

int spr_image_device_ptr(spr_handle *h, void **out) {
    if (!h || !out) return SPR_ERR_INVALID_ARG;
    if (!h->frame_valid) return SPR_ERR_NO_SCENE;
    cudaSetDevice(h->cfg.device);
    const int st = settle(h);
    if (st) return st;
    *out = h->image.p;
    return SPR_OK;
}

int spr_read_image(spr_handle *h, uint8_t *host_rgba, void *stream) {
    if (!h || !host_rgba) return SPR_ERR_INVALID_ARG;
    if (!h->frame_valid) return SPR_ERR_NO_SCENE;
    cudaSetDevice(h->cfg.device);
    const int st = settle(h);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t bytes = 4 * (size_t)h->frame_W * h->frame_H;
    if (cudaMemcpyAsync(host_rgba, h->image.p, bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess) return cuda_status();
    ++h->host_syncs;
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status();
    return SPR_OK;
}

int spr_set_output_transform(spr_handle *h, const float m[16]) {
    if (!h || !m) return SPR_ERR_INVALID_ARG;
    // 4x4 inverse by Gauss-Jordan elimination with partial pivoting (double)
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 8; ++c) a[r][c] = c < 4 ? (double)m[4 * r + c] : (c - 4 == r ? 1.0 : 0.0);
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        if (!(std::fabs(a[piv][c]) > 0.0) || !std::isfinite(a[piv][c])) return SPR_ERR_INVALID_ARG;
        if (piv != c)
            for (int k = 0; k < 8; ++k) std::swap(a[c][k], a[piv][k]);
        const double d = a[c][c];
        for (int k = 0; k < 8; ++k) a[c][k] /= d;
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            const double f = a[r][c];
            for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
        }
    }
    const int rows[3] = {0, 1, 3}, cols[3] = {0, 1, 3};
    OutputInverse inv;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            inv.m[3 * i + j] = (float)a[rows[i]][4 + cols[j]];
            if (!std::isfinite(inv.m[3 * i + j])) return SPR_ERR_INVALID_ARG;
        }
    h->out_inv = inv;
    return SPR_OK;
}

int spr_enable_output_transform(spr_handle *h, int32_t enable) {
    if (!h) return SPR_ERR_INVALID_ARG;
    h->out_tf = enable != 0;
    return SPR_OK;
}

int spr_output_device_ptr(spr_handle *h, void **out, void *stream) {
    if (!h || !out) return SPR_ERR_INVALID_ARG;
    if (!h->frame_valid) return SPR_ERR_NO_SCENE;
    cudaSetDevice(h->cfg.device);
    if (int sst = settle(h)) return sst;
    if (!h->out_tf) {
        *out = h->image.p;
        return SPR_OK;
    }
    cudaSetDevice(h->cfg.device);
    const int64_t n = (int64_t)h->frame_W * h->frame_H;
    int st = ensure(h->output, 4 * (size_t)std::max<int64_t>(n, 1));
    if (st) return st;
    launch_output_view(h->image.as<uint32_t>(), h->output.as<uint32_t>(), h->frame_W, h->frame_H, h->out_inv,
                       static_cast<cudaStream_t>(stream));
    *out = h->output.p;
    return cuda_status();
}

int spr_read_output(spr_handle *h, uint8_t *host_rgba, void *stream) {
    if (!h || !host_rgba) return SPR_ERR_INVALID_ARG;
    void *src = nullptr;
    int st = spr_output_device_ptr(h, &src, stream);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t bytes = 4 * (size_t)h->frame_W * h->frame_H;
    if (cudaMemcpyAsync(host_rgba, src, bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess) return cuda_status();
    ++h->host_syncs;
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status();
    return SPR_OK;
}

int spr_save_png(spr_handle *h, const char *path) {
    if (!h || !path) return SPR_ERR_INVALID_ARG;
    if (!h->frame_valid) return SPR_ERR_NO_SCENE;
    const int W = h->frame_W, Hh = h->frame_H;
    std::vector<uint8_t> img((size_t)W * Hh * 4), flip((size_t)W * Hh * 4);
    int st = spr_read_image(h, img.data(), nullptr);
    if (st) return st;
    // saveOutputToFile (ras_base.cpp:1221-1277): vertical flip, alpha = 255.
    for (int y = 0; y < Hh; ++y) std::memcpy(&flip[(size_t)y * W * 4], &img[(size_t)(Hh - 1 - y) * W * 4], (size_t)W * 4);
    for (size_t i = 3; i < flip.size(); i += 4) flip[i] = 255;
    return write_png_rgba(path, flip.data(), W, Hh) ? SPR_ERR_INVALID_ARG : SPR_OK;
}

int spr_get_counts(spr_handle *h, spr_element_number *out) {
    if (!h || !out) return SPR_ERR_INVALID_ARG;
    if (h->pending) {
        cudaSetDevice(h->cfg.device);
        if (int st = settle(h)) return st;
    }
    *out = h->en;
    return SPR_OK;
}

int spr_enable_step_timing(spr_handle *h, int32_t enable) {
    if (!h) return SPR_ERR_INVALID_ARG;
    h->timing = enable != 0;
    return SPR_OK;
}

int spr_step_timing(spr_handle *h, double *ms, int32_t capacity, int32_t *n_out) {
    if (!h || !n_out) return SPR_ERR_INVALID_ARG;
    *n_out = kSteps;
    if (ms)
        for (int i = 0; i < kSteps && i < capacity; ++i) ms[i] = h->step_ms[i];
    return SPR_OK;
}

int spr_debug_set_lookback(spr_handle *h, uint32_t spin_cap, int64_t hold_tile) {
    if (!h || spin_cap == 0) return SPR_ERR_INVALID_ARG;
    drop_graph(h, false);
    h->lb_spin_cap = spin_cap;
    h->lb_hold_tile = hold_tile < 0 ? -1 : hold_tile;
    return SPR_OK;
}

int spr_set_memory_limit(spr_handle *h, int64_t bytes) {
    if (!h || bytes < 0) return SPR_ERR_INVALID_ARG;
    h->budget.limit = (size_t)bytes;
    return SPR_OK;
}

int spr_get_frame_stats(spr_handle *h, spr_frame_stats *out) {
    if (!h || !out) return SPR_ERR_INVALID_ARG;
    if (h->pending) {
        cudaSetDevice(h->cfg.device);
        if (int st = settle(h)) return st;
    }
    out->kernel_launches = h->launches;
    out->host_syncs = h->host_syncs;
    out->resolve_pairs = h->npairs;
    size_t total = 0;
    for (const DevBuf *b : handle_bufs(h)) total += b->bytes;
    out->device_bytes = (int64_t)total;
    return SPR_OK;
}

const char *spr_step_name(int32_t i) { return (i >= 0 && i < kSteps) ? kStepNames[i] : nullptr; }

int spr_debug_dump(spr_handle *h, int32_t stage, void *dst, size_t capacity, size_t *needed) {
    if (!h || !needed) return SPR_ERR_INVALID_ARG;
    if (!h->frame_valid) return SPR_ERR_NO_SCENE;
    cudaSetDevice(h->cfg.device);
    if (int st = settle(h)) return st;
    const int64_t nf = h->nf;
    const int WORDS = h->frame_S / 8;
    const void *src = nullptr;
    size_t bytes = 0;
    switch (stage) {
    case SPR_STAGE_TVERTEX: src = h->tvert.p; bytes = 8 * (size_t)h->V; break;
    case SPR_STAGE_PATH_VISIBLE: src = h->pvis.p; bytes = h->P; break;
    case SPR_STAGE_CURVE_COUNT: src = h->counts.p; bytes = 4 * (size_t)h->C; break;
    case SPR_STAGE_INTERSECTION: src = h->entries.p; bytes = 8 * (size_t)nf; break;
    case SPR_STAGE_FRAG_KEY: src = h->key.p; bytes = 4 * (size_t)nf; break;
    case SPR_STAGE_FRAG_PID: src = h->pidw.p; bytes = 4 * (size_t)nf; break;
    case SPR_STAGE_FRAG_WN: src = h->wn.p; bytes = (size_t)nf; break;
    case SPR_STAGE_FRAG_MASK: src = h->mask.p; bytes = 4 * (size_t)WORDS * nf; break;
    case SPR_STAGE_SORT_PERM: src = h->perm_sorted; bytes = 4 * (size_t)nf; break;
    case SPR_STAGE_SORT_KEY: {
        bytes = 4 * (size_t)nf;
        if (nf) {
            int st = ensure(h->dump_tmp, bytes);
            if (st) return st;
            launch_decode_keys(h->skey_sorted, nf, (h->frame_H + 1) / 2, h->dump_tmp.as<int32_t>(), nullptr);
            src = h->dump_tmp.p;
        }
        break;
    }
    case SPR_STAGE_WN_SCAN: src = h->wn_scan.p; bytes = (size_t)nf; break;
    case SPR_STAGE_MERGED_MASK: src = h->merged.p; bytes = 4 * (size_t)WORDS * h->nm; break;
    case SPR_STAGE_DRAW_LIST: src = h->draw.p; bytes = 16 * (size_t)(h->nm + h->ns); break;
    case SPR_STAGE_IMAGE: src = h->image.p; bytes = 4 * (size_t)h->frame_W * h->frame_H; break;
    default: return SPR_ERR_INVALID_ARG;
    }
    *needed = bytes;
    if (!dst) return SPR_OK;  // size query
    if (capacity < bytes) return SPR_ERR_INVALID_ARG;
    if (bytes && cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) return cuda_status();
    return SPR_OK;
}

int spr_selftest(spr_handle *h, int64_t *srgb_encode_mismatches) {
    if (!h || !srgb_encode_mismatches) return SPR_ERR_INVALID_ARG;
    cudaSetDevice(h->cfg.device);
    DevBuf bad;
    int st = ensure(bad, 8);
    if (st) return st;
    cudaMemset(bad.p, 0, 8);
    launch_selftest_encode(h->rtables.as<ResolveTables>(), bad.as<unsigned long long>(), nullptr);
    unsigned long long n = 0;
    cudaMemcpy(&n, bad.p, 8, cudaMemcpyDeviceToHost);
    bad.release();
    st = cuda_status();
    *srgb_encode_mismatches = (int64_t)n;
    return st;
}

const char *spr_status_string(int32_t status) {
    switch (status) {
    case SPR_OK: return "ok";
    case SPR_ERR_INVALID_ARG: return "invalid argument";
    case SPR_ERR_INVALID_SCENE: return "invalid scene";
    case SPR_ERR_OUT_OF_MEMORY: return "out of device memory";
    case SPR_ERR_CAPACITY_EXCEEDED: return "capacity exceeded";
    case SPR_ERR_TIMEOUT: return "bounded device wait timed out";
    case SPR_ERR_CUDA: return "CUDA error";
    case SPR_ERR_NO_SCENE: return "no scene / no frame";
    case SPR_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
    }
}

}  // extern "C"

// ---- batches --------------------------------------------------------------
// A batch keeps one handle per sample count present; each handle holds the
// concatenation of its scenes (path, curve and vertex ids offset) plus the
// per-scene table, and renders all of them in one launch sequence.

constexpr int kGroups = 4;  // batch groups by sample count: 8, 16, 32, 256

struct spr_batch {
    int device = 0, ms_output = 1, srgb = 1;
    bool timing = false, graph = false;
    spr_handle *group[kGroups] = {};  // samples 8, 16, 32, 256
    // graph replays of the groups run side by side, one stream each
    cudaStream_t gstream[kGroups] = {};
    cudaEvent_t gdone[kGroups] = {}, gstart = nullptr;
    struct Entry {
        int group;
        int64_t image_off;
        int W, H;
    };
    std::vector<Entry> entries;
    bool rendered = false;
};

namespace {

int group_of(int samples) { return samples == 8 ? 0 : (samples == 16 ? 1 : (samples == 32 ? 2 : 3)); }

// Concatenates the scenes `idx` of `in` into one scene and uploads it to h,
// with the per-scene table and the scene of every path.
int upload_group(spr_handle *h, const spr_batch_scene *in, const std::vector<int> &idx,
                 std::vector<spr_batch::Entry> &entries, int g) {
    size_t P = 0, C = 0, V = 0;
    bool any_affine = false;
    for (int i : idx) {
        P += in[i].scene.n_paths;
        C += in[i].scene.n_curves;
        V += in[i].scene.n_vertices;
        any_affine |= in[i].scene.path_affine != nullptr;
    }
    if (P > (1u << 30) || C > (1u << 30) || V > (1u << 30)) return SPR_ERR_CAPACITY_EXCEEDED;
    std::vector<float> vertex(2 * V), arc_w(C, 0.f), affine(any_affine ? 6 * P : 0);
    std::vector<uint32_t> vpid(V), cvp(C), cpid(C), fill(P), pscene(P);
    std::vector<uint8_t> ctype(C), rule(P);
    std::vector<SceneInfo> info(idx.size());
    // the scenes' gradient entries and ramps, concatenated: a scene's fill
    // values 1..n_grad move by the entries before it, its entries' ramp
    // positions by the texels before it; other values below alpha 1 (which
    // draw nothing) become 0 so that they do not name another scene's entry
    std::vector<uint32_t> gtable, gramp;
    for (int i : idx) {
        if (!in[i].n_grad) continue;
        const uint32_t ebase = (uint32_t)(gtable.size() / 12), rbase = (uint32_t)gramp.size();
        if ((uint64_t)ebase + in[i].n_grad > 0x01000000u) return SPR_ERR_CAPACITY_EXCEEDED;
        gtable.insert(gtable.end(), in[i].grad_table, in[i].grad_table + 12 * (size_t)in[i].n_grad);
        for (uint32_t e = 0; e < in[i].n_grad; ++e) gtable[12 * (size_t)(ebase + e) + 6] += rbase;
        gramp.insert(gramp.end(), in[i].grad_ramp, in[i].grad_ramp + in[i].n_ramp);
    }
    uint32_t ebase = 0;
    size_t p0 = 0, c0 = 0, v0 = 0;
    int64_t pix = 0;
    uint32_t bins = 0;
    for (size_t k = 0; k < idx.size(); ++k) {
        const spr_batch_scene &b = in[idx[k]];
        const spr_scene_view &v = b.scene;
        if (v.n_vertices) std::memcpy(&vertex[2 * v0], v.vertex, 8 * (size_t)v.n_vertices);
        for (uint32_t i = 0; i < v.n_vertices; ++i) vpid[v0 + i] = v.vertex_path_id[i] + (uint32_t)p0;
        for (uint32_t i = 0; i < v.n_curves; ++i) {
            cvp[c0 + i] = v.curve_vertex_pos[i] + (uint32_t)v0;
            cpid[c0 + i] = v.curve_path_id[i] + (uint32_t)p0;
            ctype[c0 + i] = v.curve_type[i];
            if (v.curve_arc_w) arc_w[c0 + i] = v.curve_arc_w[i];
        }
        if (v.n_paths) {
            std::memcpy(&fill[p0], v.path_fill_rgba, 4 * (size_t)v.n_paths);
            std::memcpy(&rule[p0], v.path_fill_rule, v.n_paths);
        }
        if (!gtable.empty()) {
            for (uint32_t i = 0; i < v.n_paths; ++i) {
                uint32_t &f = fill[p0 + i];
                if (f >= 1u && f <= b.n_grad) f += ebase;
                else if (f < 0x01000000u) f = 0u;
            }
            ebase += b.n_grad;
        }
        for (uint32_t i = 0; i < v.n_paths; ++i) {
            pscene[p0 + i] = (uint32_t)k;
            if (any_affine) {
                static const float id6[6] = {1.f, 0.f, 0.f, 1.f, 0.f, 0.f};
                std::memcpy(&affine[6 * (p0 + i)], v.path_affine ? v.path_affine + 6 * (size_t)i : id6, 24);
            }
        }
        SceneInfo &si = info[k];
        si.W = b.width;
        si.H = b.height;
        si.ntx = (b.width + kBinW - 1) / kBinW;
        si.nrows = (b.height + 1) / 2;
        si.image_off = pix;
        si.bin_off = bins;
        si.pad = 0;
        for (int j = 0; j < 16; ++j) si.m[j] = b.has_transform ? b.transform[j] : ((j % 5 == 0) ? 1.f : 0.f);
        entries[idx[k]] = spr_batch::Entry{g, pix, b.width, b.height};
        pix += (int64_t)b.width * b.height;
        if ((int64_t)bins + (int64_t)si.ntx * si.nrows > (int64_t)UINT32_MAX) return SPR_ERR_CAPACITY_EXCEEDED;
        bins += (uint32_t)(si.ntx * si.nrows);
        p0 += v.n_paths;
        c0 += v.n_curves;
        v0 += v.n_vertices;
    }
    spr_scene_view cat{(uint32_t)P,    (uint32_t)C,  (uint32_t)V,  vertex.data(), vpid.data(), cvp.data(),
                       ctype.data(),   cpid.data(),  arc_w.data(), rule.data(),   fill.data(),
                       any_affine ? affine.data() : nullptr};
    int st = spr_set_scene(h, &cat);
    if (st) return st;
    if ((st = upload(h->scenes_d, info.data(), info.size())) || (st = upload(h->path_scene, pscene.data(), P)))
        return st;
    if ((st = spr_set_gradients(h, gtable.empty() ? nullptr : gtable.data(), (uint32_t)(gtable.size() / 12),
                                gramp.empty() ? nullptr : gramp.data(), (uint32_t)gramp.size())))
        return st;
    h->scenes_h = info;
    h->scenes_shift = kBinShift;
    h->n_scenes = (int)info.size();
    return SPR_OK;
}

}  // namespace

extern "C" {

int spr_batch_create(int32_t device, int32_t ms_output, int32_t srgb, spr_batch **out) {
    if (!out) return SPR_ERR_INVALID_ARG;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return cuda_status();
    spr_batch *b = new (std::nothrow) spr_batch();
    if (!b) return SPR_ERR_OUT_OF_MEMORY;
    b->device = device;
    b->ms_output = ms_output ? 1 : 0;
    b->srgb = srgb ? 1 : 0;
    *out = b;
    return SPR_OK;
}

int spr_batch_destroy(spr_batch *b) {
    if (!b) return SPR_OK;
    for (spr_handle *&h : b->group) {
        spr_destroy(h);
        h = nullptr;
    }
    for (int g = 0; g < kGroups; ++g) {
        if (b->gstream[g]) cudaStreamDestroy(b->gstream[g]);
        if (b->gdone[g]) cudaEventDestroy(b->gdone[g]);
    }
    if (b->gstart) cudaEventDestroy(b->gstart);
    delete b;
    return SPR_OK;
}

int spr_batch_set_scenes(spr_batch *b, const spr_batch_scene *scenes, int32_t n) {
    if (!b || n < 0 || (n > 0 && !scenes)) return SPR_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i) {
        const spr_batch_scene &s = scenes[i];
        if (s.width < 1 || s.height < 1 || s.width > 4096 || s.height > 4096) return SPR_ERR_INVALID_ARG;
        if (s.samples != 8 && s.samples != 16 && s.samples != 32 && s.samples != 256) return SPR_ERR_INVALID_ARG;
        if (s.samples == 256 && !b->ms_output) return SPR_ERR_INVALID_ARG;
        int st = validate_scene(&s.scene);
        if (st) return st;
        if (s.n_grad && (st = check_gradients(s.grad_table, s.n_grad, s.grad_ramp, s.n_ramp))) return st;
    }
    cudaSetDevice(b->device);
    b->rendered = false;
    b->entries.assign(n, spr_batch::Entry{0, 0, 0, 0});
    std::vector<int> idx[kGroups];
    for (int i = 0; i < n; ++i) idx[group_of(scenes[i].samples)].push_back(i);
    for (int g = 0; g < kGroups; ++g) {
        if (idx[g].empty()) {
            spr_destroy(b->group[g]);
            b->group[g] = nullptr;
            continue;
        }
        if (!b->group[g]) {
            const spr_config cfg{scenes[idx[g][0]].width, scenes[idx[g][0]].height, scenes[idx[g][0]].samples,
                                 b->ms_output, b->srgb, b->device};
            int st = spr_create(&cfg, &b->group[g]);
            if (st) return st;
            b->group[g]->timing = b->timing;
            b->group[g]->graph_mode = b->graph;
        }
        int st = upload_group(b->group[g], scenes, idx[g], b->entries, g);
        if (st) return st;
    }
    return SPR_OK;
}

namespace {
// Graph replay of every group at once: each group's captured frame on its
// own stream, ordered after the caller's stream and joined back into it.
// Returns false (nothing launched) unless every group has a current graph.
bool replay_groups_concurrently(spr_batch *b, cudaStream_t s) {
    int n = 0;
    for (spr_handle *h : b->group) {
        if (!h) continue;
        if (!h->graph_mode || h->timing || !h->gexec || h->gexec_gen != g_alloc_gen.load() || !h->caps_ok) return false;
        ++n;
    }
    if (n < 2) return false;
    cudaSetDevice(b->device);
    if (!b->gstart && cudaEventCreateWithFlags(&b->gstart, cudaEventDisableTiming) != cudaSuccess) return false;
    for (int g = 0; g < kGroups; ++g) {
        if (!b->group[g]) continue;
        if (!b->gstream[g] && cudaStreamCreateWithFlags(&b->gstream[g], cudaStreamNonBlocking) != cudaSuccess)
            return false;
        if (!b->gdone[g] && cudaEventCreateWithFlags(&b->gdone[g], cudaEventDisableTiming) != cudaSuccess) return false;
    }
    cudaEventRecord(b->gstart, s);
    for (int g = 0; g < kGroups; ++g) {
        spr_handle *h = b->group[g];
        if (!h) continue;
        cudaStreamWaitEvent(b->gstream[g], b->gstart, 0);
        supersede(h);
        cudaGraphLaunch(h->gexec, b->gstream[g]);
        mark_pending(h, b->gstream[g]);
        cudaEventRecord(b->gdone[g], b->gstream[g]);
        cudaStreamWaitEvent(s, b->gdone[g], 0);
        h->host_syncs = 0;
        h->frame_valid = true;
        ++h->graph_replays;
    }
    return true;
}
}  // namespace

int spr_batch_render(spr_batch *b, void *stream) {
    if (!b) return SPR_ERR_INVALID_ARG;
    if (b->entries.empty()) return SPR_ERR_NO_SCENE;
    b->rendered = false;
    if (b->graph && replay_groups_concurrently(b, static_cast<cudaStream_t>(stream))) {
        const int st = cuda_status();
        if (st) return st;
        b->rendered = true;
        return SPR_OK;
    }
    for (spr_handle *h : b->group) {
        if (!h) continue;
        int st = spr_render(h, stream);
        if (st) return st;
    }
    b->rendered = true;
    return SPR_OK;
}

namespace {
// Every group's frame settled (see settle()).
int settle_batch(spr_batch *b) {
    cudaSetDevice(b->device);
    for (spr_handle *h : b->group)
        if (h && h->pending)
            if (int st = settle(h)) return st;
    return SPR_OK;
}
}  // namespace

int spr_batch_image_device_ptr(spr_batch *b, int32_t scene, void **out) {
    if (!b || !out || scene < 0 || scene >= (int32_t)b->entries.size()) return SPR_ERR_INVALID_ARG;
    if (!b->rendered) return SPR_ERR_NO_SCENE;
    if (int st = settle_batch(b)) return st;
    const spr_batch::Entry &e = b->entries[scene];
    *out = b->group[e.group]->image.as<uint32_t>() + e.image_off;
    return SPR_OK;
}

int spr_batch_read_image(spr_batch *b, int32_t scene, uint8_t *host_rgba, void *stream) {
    if (!b || !host_rgba || scene < 0 || scene >= (int32_t)b->entries.size()) return SPR_ERR_INVALID_ARG;
    if (!b->rendered) return SPR_ERR_NO_SCENE;
    if (int st = settle_batch(b)) return st;
    cudaSetDevice(b->device);
    const spr_batch::Entry &e = b->entries[scene];
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t *src = b->group[e.group]->image.as<uint32_t>() + e.image_off;
    if (cudaMemcpyAsync(host_rgba, src, 4 * (size_t)e.W * e.H, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return cuda_status();
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status();
    return SPR_OK;
}

int spr_batch_get_counts(spr_batch *b, spr_element_number *total) {
    if (!b || !total) return SPR_ERR_INVALID_ARG;
    if (int st = settle_batch(b)) return st;
    spr_element_number t{};
    for (spr_handle *h : b->group) {
        if (!h) continue;
        t.path += h->en.path;
        t.curve += h->en.curve;
        t.vertex += h->en.vertex;
        t.curve_fragment += h->en.curve_fragment;
        t.merged_fragment += h->en.merged_fragment;
        t.span += h->en.span;
    }
    *total = t;
    return SPR_OK;
}

namespace {
// The one group handle of a batch whose scenes share a sample count (its
// concatenation order is the scene order), else null.
spr_handle *single_group(spr_batch *b) {
    spr_handle *one = nullptr;
    for (spr_handle *h : b->group) {
        if (!h) continue;
        if (one) return nullptr;
        one = h;
    }
    return one;
}
}  // namespace

int spr_batch_diff_render(spr_batch *b, const float *fill_rgba, float *image, void *stream) {
    if (!b || !fill_rgba || !image) return SPR_ERR_INVALID_ARG;
    if (b->entries.empty()) return SPR_ERR_NO_SCENE;
    spr_handle *h = single_group(b);
    if (!h) return SPR_ERR_UNSUPPORTED;
    b->rendered = false;
    const DiffCall dc{false, fill_rgba, nullptr, image, nullptr, nullptr, nullptr};
    return frame(h, stream, &dc);
}

int spr_batch_diff_backward(spr_batch *b, const float *fill_rgba, const float *grad_image, float *grad_fill,
                            float *grad_vertex, float *grad_affine, void *stream) {
    if (!b || !fill_rgba || !grad_image || !grad_fill || !grad_vertex) return SPR_ERR_INVALID_ARG;
    if (b->entries.empty()) return SPR_ERR_NO_SCENE;
    spr_handle *h = single_group(b);
    if (!h) return SPR_ERR_UNSUPPORTED;
    if (grad_affine && !h->has_affine) return SPR_ERR_INVALID_ARG;
    b->rendered = false;
    const DiffCall dc{true, fill_rgba, grad_image, nullptr, grad_fill, grad_vertex, grad_affine};
    return backward_frame(h, stream, dc);
}

int spr_batch_update_vertices(spr_batch *b, const float *vertex, void *stream) {
    if (!b || !vertex) return SPR_ERR_INVALID_ARG;
    if (b->entries.empty()) return SPR_ERR_NO_SCENE;
    spr_handle *h = single_group(b);
    if (!h) return SPR_ERR_UNSUPPORTED;
    b->rendered = false;
    return spr_update_vertices(h, vertex, stream);
}

int spr_batch_set_graph_replay(spr_batch *b, int32_t enable) {
    if (!b) return SPR_ERR_INVALID_ARG;
    b->graph = enable != 0;
    for (spr_handle *h : b->group)
        if (h) spr_set_graph_replay(h, enable);
    return SPR_OK;
}

int spr_batch_enable_step_timing(spr_batch *b, int32_t enable) {
    if (!b) return SPR_ERR_INVALID_ARG;
    b->timing = enable != 0;
    for (spr_handle *h : b->group)
        if (h) h->timing = b->timing;
    return SPR_OK;
}

int spr_batch_step_timing(spr_batch *b, double *ms, int32_t capacity, int32_t *n_out) {
    if (!b || !n_out) return SPR_ERR_INVALID_ARG;
    *n_out = kSteps;
    if (ms)
        for (int i = 0; i < kSteps && i < capacity; ++i) {
            ms[i] = 0.0;
            for (spr_handle *h : b->group)
                if (h) ms[i] += h->step_ms[i];
        }
    return SPR_OK;
}

int spr_batch_get_frame_stats(spr_batch *b, spr_frame_stats *out) {
    if (!b || !out) return SPR_ERR_INVALID_ARG;
    spr_frame_stats t{};
    for (spr_handle *h : b->group) {
        if (!h) continue;
        spr_frame_stats f{};
        spr_get_frame_stats(h, &f);
        t.kernel_launches += f.kernel_launches;
        t.host_syncs += f.host_syncs;
        t.resolve_pairs += f.resolve_pairs;
        t.device_bytes += f.device_bytes;
    }
    *out = t;
    return SPR_OK;
}

}  // extern "C"
