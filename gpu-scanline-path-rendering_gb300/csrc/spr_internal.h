// spr_internal.h -- declarations shared by the host orchestration
// (spr_api.cpp) and the CUDA translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace spr {

// Per-curve descriptor, one 16-byte load per curve.
struct CurveDesc {
    uint32_t vpos;  // first control point
    uint32_t pid;   // path id
    float w;        // rational weight (0 for other types)
    uint32_t type;  // curve type | reversed << 8
};

// Device-resident lookup tables of the resolve: sRGB decode, linear decode,
// encode thresholds and the 4096-bin encode base.
struct ResolveTables {
    float srgb_dec[256];
    float lin_dec[256];
    float threshold[256];  // 255 used
    uint8_t bin[4096];
};

// Frame status bits (FrameCounters::status).
constexpr uint32_t kStatusOverflow = 1u;  // a frame size exceeded its buffers
constexpr uint32_t kStatusTimeout = 2u;   // a bounded device wait gave up
// Polls of a look-back window before it gives up: about a second of waiting
// (each poll sleeps 64 ns at least), far beyond any real wait.
constexpr uint32_t kLbSpinCap = 1u << 24;

// Frame-level sizes and flags written by the kernels (device memory): a
// frame's kernels read their sizes here, so no size has to come back to the
// host.  A size is "admitted" once it is known to fit its buffers; one that
// does not fit is admitted as 0 (the rest of the frame then does nothing)
// and sets kStatusOverflow, and the frame is rendered again with larger
// buffers before anything reads it.
struct FrameCounters {
    uint32_t n_merged;     // merged fragments (draw items with sample masks)
    uint32_t n_span;       // spans
    uint32_t n_pairs;      // resolve pairs, admitted
    uint32_t status;       // kStatusOverflow | kStatusTimeout
    uint32_t bin_queue;    // next resolve bin to hand out (persistent resolve)
    uint32_t nf;           // intersection entries, admitted
    uint32_t need_nf;      // intersection entries of the frame
    uint32_t need_pairs;   // resolve pairs of the frame
    uint32_t n_items;      // n_merged + n_span
    uint32_t tiles[3];     // look-back tile counters: entry offsets, scan-mark, pair offsets
    uint32_t diff_status;  // differentiable frames: bit 0 tape too short, bit 1 chain too short
    uint32_t pairs_alt;          // resolve pairs in the other built-in tile (FrameArgs::alt_shift)
    unsigned long long span_px;  // the spans' pixels (sum of their widths)
};

// Resolve bins: a bin is a band of 64 / bin_w cell rows x bin_w pixel
// columns holding 32 cells (one per lane of the warp that resolves it),
// bin_w = 1 << shift, shift 3..6 (8 x 8, 16 x 4, 32 x 2 or 64 x 1 cells).
// Plain frames use 16 x 4 when their spans are short (at most
// kShortSpanPx pixels of span per draw item, measured by the sized frame:
// narrower tiles cut long spans into many more pairs), else 64 x 1, unless
// the tuning picks a tile; differentiable frames use 64 x 1 (kBinW columns,
// one cell row).
constexpr int kBinW = 64;
constexpr int kBinShift = 6;
constexpr int kPlainBinShift = 4;
constexpr int kShortSpanPx = 8;
__host__ __device__ __forceinline__ int bin_cols(int W, int shift) { return (W + (1 << shift) - 1) >> shift; }
__host__ __device__ __forceinline__ int bin_rows(int H, int shift) {
    const int band_shift = kBinShift - shift;  // cell rows per band: 1 << band_shift
    return (((H + 1) / 2) + (1 << band_shift) - 1) >> band_shift;
}
// One scene of a batch frame: its viewport, its resolve bins (ntx tiles x
// nrows bands of the frame's bin geometry, numbered from bin_off) and its
// image (W x H
// pixels from image_off in the frame's image buffer), and its 4x4 input
// transform (row-major).
struct SceneInfo {
    int32_t W, H;
    int32_t ntx, nrows;
    int64_t image_off;
    uint32_t bin_off;
    uint32_t pad;
    float m[16];
};

// ---- host-built tables (spr_tables.cpp) --------------------------------------
// Cell sample positions, float2[4 * samples] (pixel k = px.x*2 + px.y).
void build_cell_samples(int samples, float *out);
// 256x256 half-plane mask table, uint32[65536 * samples/8].
void build_mask_table(int samples, uint32_t *out);
// 256-sample frames are 8 passes of 32 samples: pass g covers rows 8j + g of
// the 256-row pattern with the 32-sample rows and its own mask table
// (uint32[65536 * 4]), the geometry moved by -pass_shift_256(g) pixel in y.
constexpr int kPasses256 = 8;
void build_pass_mask_table_256(int pass, uint32_t *out);
float pass_shift_256(int pass);
void build_resolve_tables(ResolveTables *t);

// ---- scan / sort (spr_sort.cu) ----------------------------------------------------
int64_t scan_tmp_words(int64_t n);
// Single-pass exclusive scan (decoupled look-back) of n u32 values:
// out[0..n) = exclusive prefix sums, out[n] = total, *total_out = total when
// given.  n = *n_dev when n_dev is given (at most n_cap: the grid is sized
// for n_cap), else n_cap.  tile_status holds lookback_words(n_cap) words and
// *tile_ctr one word, both zero before the call.  A wait longer than
// spin_cap polls sets kStatusTimeout in *frame_status.  in and out must be
// 16-byte aligned.  hold_tile >= 0 (tests of the timeout only): that tile
// never publishes, so the tiles after it wait until spin_cap runs out.
int64_t lookback_words(int64_t n);
int scan_lookback_u32(const uint32_t *in, uint32_t *out, const uint32_t *n_dev, int64_t n_cap, uint64_t *tile_status,
                      uint32_t *tile_ctr, uint32_t spin_cap, uint32_t *frame_status, uint32_t *total_out,
                      cudaStream_t s, int64_t hold_tile = -1);
// Admits a size: *admitted = *need if *need <= cap, else 0 and
// kStatusOverflow in *status; 0 as well after a timeout (the size may be
// wrong then).
int launch_admit(const uint32_t *need, uint32_t *admitted, uint32_t cap, uint32_t *status, cudaStream_t s);
// out[0..n) = exclusive prefix sums of in, out[n] = total.
int scan_exclusive_u32(const uint32_t *in, uint32_t *out, int64_t n, uint32_t *tmp, cudaStream_t s);
// In-place exclusive scan of a short array by one block; a[n] = total.
int scan_tiles_inplace(uint32_t *a, int64_t n, cudaStream_t s);
int64_t radix_tiles(int64_t n);
// Stable sort of the fragment entries by (path, 24-bit cell key), given that
// they arrive grouped by path: every path's segment sorted by one block.
// Reads keys (values are the positions), writes keys_out / vals_out; keys and
// vals serve as scratch for long segments.  path_start: P + 1 words.
// Nothing is sorted when the frame's entries were not admitted (ctr->nf 0).
// Sort key of a fragment: path << 24 | cell key within the path (24 bits),
// with the fragment's scan winding swn and change sign chg (each -1, 0 or
// 1) carried in bits 60-63 (pack_fw), above every bit the sorts order by.
// Readers that compare keys mask them with kKeyMask.
constexpr int kFwShift = 60;
constexpr uint64_t kKeyMask = (1ull << kFwShift) - 1ull;
__host__ __device__ __forceinline__ uint32_t pack_fw(int swn, int chg) {
    return (uint32_t)((swn & 3) | ((chg & 3) << 2));
}
__host__ __device__ __forceinline__ int fw_swn(uint32_t b) { return (int)(b << 30) >> 30; }
__host__ __device__ __forceinline__ int fw_chg(uint32_t b) { return (int)(b << 28) >> 30; }
int launch_segment_sort(const CurveDesc *curves, uint32_t C, uint32_t P, const uint32_t *offsets, uint64_t *keys,
                        uint32_t *vals, uint64_t *keys_out, uint32_t *vals_out, uint32_t *path_start,
                        const FrameCounters *ctr, cudaStream_t s);
int64_t radix_tmp_words(int64_t n);
// Stable LSD sort on bits [0, key_bits); returns true when the result is in
// the *_alt buffers.
// *launches receives the number of kernels launched.
// n = *n_dev when n_dev is given (at most n: the grids are sized for n).
template <class K>
bool radix_sort(K *keys, uint32_t *vals, K *keys_alt, uint32_t *vals_alt, int64_t n, int key_bits, uint32_t *tmp,
                cudaStream_t s, int *launches, const uint32_t *n_dev = nullptr);

// ---- pipeline kernels (spr_kernels.cu); each launcher returns its kernel count --
struct FrameArgs {
    int W, H, S, ms_output, srgb;
    int P, C, V;
    float m[16];
    // scene
    const float2 *vertex;
    const uint32_t *vertex_pid;
    const float *affine;  // nullable
    const CurveDesc *curves;
    const uint8_t *fill_rule;
    const uint32_t *fill_rgba;
    const uint32_t *mask_table;
    const ResolveTables *rtables;
    // Batch frames: path p belongs to scenes[path_scene[p]], whose viewport,
    // transform and image replace W, H and m above.  Both are null for a
    // single-scene frame.
    const uint32_t *path_scene;
    const SceneInfo *scenes;
    int n_scenes;
    int64_t n_bins;  // resolve bins of the frame
    int bin_shift;   // bins of 1 << bin_shift pixel columns x 64 >> bin_shift cell rows
    int alt_shift;   // the other built-in tile, whose pairs the scan-mark pass also counts (-1: none)
    // Differentiable frames (else null): per fragment its chord in cell
    // units (q0, q1) and its left mask; per draw item its path.
    float4 *chord;
    uint32_t *lmask;
    uint32_t *vmask;  // rows between the chord's end points (vertical_mask2)
    uint32_t *item_path;
    // Passes of a 256-sample frame (else 0 and null): the geometry's shift
    // down the pixel (subtracted from transformed y), and the per-pixel
    // fixed-point sample sums (4 per pixel) that the resolve adds its pass to.
    float pass_dy;
    long long *sums;
    // Gradient paints (else null): 3 float4 per entry (fill value - 1), the
    // RGBA8 ramp texels in rows of 1024, and the reverse transform
    // (rx, ry, rw, rp, a) from pixel to scene coordinates.
    const float4 *grad_table;
    uint32_t n_grad;
    const uint32_t *grad_ramp;
    float rev[13];
    int resolve_bps;  // resolve blocks per SM (1..4; 0 = the default 4)
};

int launch_transform(const FrameArgs &a, float2 *tvert, uint32_t *path_flags, uint8_t *path_visible,
                      cudaStream_t s);
int launch_curve_count(const FrameArgs &a, const float2 *tvert, const uint8_t *path_visible, uint32_t *counts,
                        cudaStream_t s);
// Sort keys of the emission order (curves by decreasing estimated cost).
int launch_emit_keys(const FrameArgs &a, const uint32_t *counts, uint32_t *key, uint32_t *val, cudaStream_t s);
// order: curve processed by thread i (null = identity); outputs do not depend on it.
// The kernels below read the frame's sizes from the counters (ctr); their
// grids are sized for the buffers' capacities (cap_*).
int launch_curve_emit(const FrameArgs &a, const float2 *tvert, const uint8_t *path_visible,
                      const uint32_t *offsets, const uint32_t *order, int2 *entries, const FrameCounters *ctr,
                      cudaStream_t s);
int launch_fragment(const FrameArgs &a, const float2 *tvert, const int2 *entries, int64_t cap_nf,
                    const FrameCounters *ctr, int32_t *key, uint32_t *pidw, int8_t *wn, uint32_t *mask,
                    uint64_t *sort_key, uint32_t *sort_val, cudaStream_t s);
// Look-back words of launch_scan_mark (zero before the launch).
int64_t scan_mark_status_words(int64_t cap_nf);
// Winding scan, merged-fragment / span marks, draw list and merged heads in
// one pass (decoupled look-back); writes the item counts to the counters
// and adds every item's pairs to bin_count (n_bins words, zero before).
// item_scene (batch frames only, else null) receives the scene of each draw
// item; in batch frames the winding scan restarts at every scene.
int launch_scan_mark(const FrameArgs &a, int64_t cap_nf, const uint64_t *skey, int8_t *wn_scan, int4 *draw,
                     uint32_t *heads, uint32_t *item_scene, uint32_t *bin_count, FrameCounters *counters,
                     uint64_t *tile_status, uint32_t spin_cap, cudaStream_t s);
// Merged masks from the sorted keys and fragment indices (perm), which hold
// at least 16 entries past cap_nf, and the fragments' masks.
int launch_stencil(const FrameArgs &a, int64_t cap_nf, FrameCounters *ctr, const uint64_t *skey, const uint32_t *perm,
                   const uint32_t *mask, const int8_t *wn_scan, const uint32_t *heads, uint32_t *merged_mask,
                   uint32_t spin_cap, cudaStream_t s);
// The draw items of every resolve bin in draw order: bin b's are
// pval[bin_off[b] .. bin_off[b + 1]) (bin_off: the exclusive scan of the
// bin counts; bin_fill: n_bins words, zero before).
int launch_bin_scatter(const FrameArgs &a, const int4 *draw, const uint32_t *item_scene, int64_t cap_items,
                       const FrameCounters *ctr, const uint32_t *bin_off, uint32_t *bin_fill, uint32_t *pval,
                       cudaStream_t s);
// Pairs of every bin counted from the draw list into bin_count (zero before).
int launch_bin_count(const FrameArgs &a, const int4 *draw, const uint32_t *item_scene, int64_t cap_items,
                     const FrameCounters *ctr, uint32_t *bin_count, cudaStream_t s);
// Sorts every bin's item indices into draw order.  With rec_a set, also
// writes the resolve records in that order: rec_a[p] = (colour, first
// column | width << 16 | cell row within the bin's band << 29) and rec_m[p]
// the sample mask (S / 8 words; every sample for a span).
int launch_bin_sort(const uint32_t *bin_off, int64_t nbins, uint32_t *pval, const FrameCounters *ctr, int S,
                    int bin_shift, const int4 *draw, const uint32_t *merged, uint2 *rec_a, uint32_t *rec_m,
                    cudaStream_t s);
// The resolve is persistent: resolve_warps(a) warps take bins from
// counters->bin_queue (zeroed by launch_resolve).  overflow:
// resolve_overflow_words(a) words, the cell entries past the ones each warp
// keeps in shared memory (multisample modes; unused otherwise).
int64_t resolve_warps(const FrameArgs &a);
int64_t resolve_overflow_words(const FrameArgs &a);
// RGBA8 image of a 256-sample frame from the sums its 8 passes accumulated.
// Rows 0, 1 and 3 (columns 0, 1, 3) of the output transform's inverse.
struct OutputInverse {
    float m[9];
};
int launch_output_view(const uint32_t *image, uint32_t *out, int W, int H, const OutputInverse &inv, cudaStream_t s);
int launch_encode_sums(const FrameArgs &a, const long long *sums, uint32_t *image, int64_t npix, cudaStream_t s);
int launch_resolve(const FrameArgs &a, const uint2 *rec_a, const uint32_t *rec_m, const uint32_t *bin_start,
                   const uint32_t *bin_end, uint32_t *image, uint32_t *overflow, FrameCounters *counters,
                   cudaStream_t s);
int launch_fill(uint32_t *image, int64_t n, uint32_t value, cudaStream_t s);
// Scene upload on the device: validation, curve orientation (vertices
// reversed in place), curve descriptors, the stored -> input vertex map.
// flags (zeroed by the caller): bit 0 invalid scene, bit 1 overlapping or
// unordered curve vertex ranges.
int launch_scene_prepare(const uint32_t *cvp, const uint8_t *ctype, const uint32_t *cpid, const float *arcw,
                         uint32_t C, uint32_t V, uint32_t P, float2 *vert, const uint32_t *vpid, uint32_t *vmap,
                         CurveDesc *cd, uint32_t *flags, cudaStream_t s);
int launch_selftest_encode(const ResolveTables *rt, unsigned long long *bad, cudaStream_t s);
int launch_decode_keys(const uint64_t *skey, int64_t nf, int nrows, int32_t *out, cudaStream_t s);

// Differentiable frames (spr_diff.cu).  Device pointers; fill is linear
// RGBA per path.  Gradients are accumulated (the caller zeroes them).
struct DiffArgs {
    const float4 *fill;
    const float4 *grad_image;  // backward input, dL/d(pixel), W x H
    float4 *image;             // forward output, W x H
    float4 *grad_fill;         // per path
    float2 *grad_tvert;        // per stored vertex, in transformed space
    const int4 *draw;
    const uint32_t *merged;
    const uint32_t *pval, *bstart, *bend;
    int64_t npairs;
    // the resolve pairs' items gathered in bin order: (pos, length, merged
    // index + 1, path), the path's fill, the merged sample mask
    uint4 *bitem;
    float4 *bfill;
    uint4 *bmm;
    const float4 *chord;
    const uint32_t *lmask, *vmask, *pidw, *perm, *heads, *item_path;
    // per fragment crossing sums (raw fragment, slope, sum dL/dx (1 - lam),
    // sum dL/dx lam), chained to the control points by a second kernel
    float4 *chain;
    uint32_t *n_chain;
    const uint64_t *skey;
    const int8_t *wn_scan;
    const int2 *entries;
    const float2 *tvert;
    int64_t nf;
    float4 *tape;      // per block: tape_depth x (samples per thread) x block threads (sample states)
    float4 *tape_rec;  // per block: warps x tape_depth x 3 (per-cell item records)
    int tape_depth;
    uint32_t *queue;     // bin queue (zeroed by the launchers)
    uint32_t *status;    // bit 0: a tape overflowed (rerun with a deeper tape); bit 1: chain list full
    // pixel = out_scale * (mean of the samples), added to the image when
    // accumulate (the passes of a 256-sample frame: 1/8 each); the backward
    // takes out_scale * dL/d(pixel) likewise
    float out_scale;
    int accumulate;
};
int64_t diff_blocks(const FrameArgs &a);
int64_t diff_tape_words(const FrameArgs &a, int depth);      // float4 count of the sample-state tape
int64_t diff_tape_rec_words(const FrameArgs &a, int depth);  // float4 count of the item records
int launch_diff_forward(const FrameArgs &a, const DiffArgs &d, cudaStream_t s);
int launch_diff_backward(const FrameArgs &a, const DiffArgs &d, cudaStream_t s);
// dL/d(stored vertex in transformed space) -> dL/d(input vertex), dL/d(path affine).
// vmap: stored vertex -> input vertex index (curves reversed on upload).
int launch_diff_vertex(const FrameArgs &a, const float2 *grad_tvert, const uint32_t *vmap, float2 *grad_vertex,
                       float *grad_affine, cudaStream_t s);
// dst = src (first) or dst + src, n floats.
int launch_accumulate(float *dst, const float *src, int64_t n, int first, cudaStream_t s);

}  // namespace spr
