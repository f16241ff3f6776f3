/*
 * spr.h -- C ABI of the GB300-native scanline path renderer.
 *
 * This header is the drop-in boundary for the reference's rasterizer plugin
 * interface, the abstract C++ class RasterizerBase::VGRasterizer
 * (gpu-scanline/src/rasterizer/shared/ras_base.h:133-378) created through
 * createRasterizer(PM_Cut_Mask_Comb_Scanline)
 * (gpu-scanline/src/rasterizer/shared/ras_factory.h:18-34).  Every entry point
 * below names the reference member it replaces.  The signatures use plain C
 * types only (no CUDA, no torch): a CUDA stream is passed as `void *`
 * (a cudaStream_t, NULL = the legacy default stream).
 *
 * Differences from the reference boundary, by design:
 *   - errors are returned as status codes instead of C++ exceptions;
 *   - saving the output never calls exit() (ras_base.cpp:1276);
 *   - there is no OpenGL: the output is an RGBA8 image in device memory that
 *     the caller can read back or write to a PNG file.
 */
#ifndef SPR_H_
#define SPR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum spr_status {
    SPR_OK = 0,
    SPR_ERR_INVALID_ARG = 1,       /* bad pointer, size or option            */
    SPR_ERR_INVALID_SCENE = 2,     /* bad curve type, index or path order    */
    SPR_ERR_OUT_OF_MEMORY = 3,     /* device allocation failed               */
    SPR_ERR_CAPACITY_EXCEEDED = 4, /* a fixed-capacity buffer overflowed     */
    SPR_ERR_TIMEOUT = 5,           /* a bounded device wait gave up          */
    SPR_ERR_CUDA = 6,              /* any other CUDA runtime error           */
    SPR_ERR_NO_SCENE = 7,          /* render called before spr_set_scene     */
    SPR_ERR_UNSUPPORTED = 8        /* option not supported by this library   */
};

/* ---- scene model ------------------------------------------------------- */
/* Curve type codes; the low 3 bits are the control-point count
 * (gpu-scanline/src/bezier_curve_type.h:6-18). */
enum spr_curve_type {
    SPR_CURVE_LINEAR = 0x02,
    SPR_CURVE_QUADRATIC = 0x03,
    SPR_CURVE_CUBIC = 0x04,
    SPR_CURVE_RATIONAL = 0x13
};

/* Fill rules (gpu-scanline/src/vg_container.h:43-46). */
enum spr_fill_rule { SPR_FILL_NONZERO = 0, SPR_FILL_EVEN_ODD = 1 };

/*
 * Flat structure-of-arrays scene, the same layout as the reference's
 * VGInputCurveDataPack / VGInputPathDataPack (ras_base.h:34-112) filled by
 * addVg (ras_base.cpp:70-382).  All pointers are HOST pointers.
 *
 *   vertex            float2[n_vertices] (x, y interleaved).  Vertices are not
 *                     shared: curve i owns (curve_type[i] & 7) consecutive
 *                     vertices starting at curve_vertex_pos[i].
 *   vertex_path_id    uint32[n_vertices], path of each vertex.
 *   curve_vertex_pos  uint32[n_curves].
 *   curve_type        uint8[n_curves], one of spr_curve_type.
 *   curve_path_id     uint32[n_curves], non-decreasing (curves are grouped
 *                     by path, in painter's order).
 *   curve_arc_w       float[n_curves], middle weight of rational curves
 *                     (ignored for other types); may be NULL if the scene has
 *                     no rational curve.
 *   path_fill_rule    uint8[n_paths], spr_fill_rule.
 *   path_fill_rgba    uint32[n_paths], solid colour r | g<<8 | b<<16 | a<<24.
 *                     A colour with a = 0 is stored as 0 (ras_base.cpp:148-152).
 *   path_affine       optional float[6 * n_paths]: per-path affine
 *                     (a, b, c, d, e, f): x' = a*x + c*y + e, y' = b*x + d*y + f,
 *                     applied before the global transform.  NULL = identity.
 *                     (The reference bakes path transforms into vertices in
 *                     its loader, rvg.cpp:400-431; here it is a device-side
 *                     stage so that it can be differentiated.)
 */
typedef struct spr_scene_view {
    uint32_t n_paths;
    uint32_t n_curves;
    uint32_t n_vertices;
    const float *vertex;
    const uint32_t *vertex_path_id;
    const uint32_t *curve_vertex_pos;
    const uint8_t *curve_type;
    const uint32_t *curve_path_id;
    const float *curve_arc_w;
    const uint8_t *path_fill_rule;
    const uint32_t *path_fill_rgba;
    const float *path_affine;
} spr_scene_view;

/* ---- renderer configuration ------------------------------------------- */
/*
 * width, height : output buffer size, 1..4096 each (resizeOutputBuffer,
 *                 ras_base.cpp:396-402; the reference caps its buffers at
 *                 4096, ras_define.h:17-20).
 * samples       : samples per pixel, 8 or 32 (setSamples), or 16 or 256 (an
 *                 extension: the 8-sample bit-reversal pattern on 16 or 256
 *                 rows).  A 256-sample frame is rendered as 8 passes of 32
 *                 samples (pass g: rows 8j + g, the geometry moved up by
 *                 (2g - 7) / 512 pixel so that they fall on the 32-sample
 *                 rows); its pixels are the exact means of all 256 samples.
 *                 256 samples need ms_output = 1.  Counts and stage dumps of
 *                 a 256-sample frame are those of its last pass.
 * ms_output     : 1 = per-sample coverage resolve (the reference's
 *                 multisample GL output, setMultisampleOutput); 0 = one colour
 *                 per pixel with alpha scaled by coverage.
 * srgb          : 1 = sRGB-correct blending (enableSRGBCorrection).
 * device        : CUDA device ordinal.
 */
typedef struct spr_config {
    int32_t width;
    int32_t height;
    int32_t samples;
    int32_t ms_output;
    int32_t srgb;
    int32_t device;
} spr_config;

/* Element counts of the last frame (ElementNumber, ras_base.h:124-131). */
typedef struct spr_element_number {
    int32_t path;
    int32_t curve;
    int32_t vertex;
    int32_t curve_fragment;
    int32_t merged_fragment;
    int32_t span;
} spr_element_number;

typedef struct spr_handle spr_handle;

/* ---- lifetime ---------------------------------------------------------- */
/* createRasterizer + VGRasterizer::init (ras_factory.h:18-34,
 * ras_cut_mask_comb_scanline.cpp:31-45): builds the sample pattern and the
 * half-plane mask table and uploads them to the device. */
int spr_create(const spr_config *config, spr_handle **out);
/* VGRasterizer::uninit / destructor. Accepts NULL. */
int spr_destroy(spr_handle *h);

/* resizeOutputBuffer (ras_base.cpp:396-402). */
int spr_resize(spr_handle *h, int32_t width, int32_t height);
/* setSamples (ras_base.h:185); 8, 16, 32 or 256.  Rebuilds the device tables. */
int spr_set_samples(spr_handle *h, int32_t samples);
/* setMultisampleOutput (ras_base.h:186); SPR_ERR_INVALID_ARG to turn it off
 * at 256 samples. */
int spr_set_multisample_output(spr_handle *h, int32_t enable);
/* enableSRGBCorrection (ras_base.h:179). */
int spr_enable_srgb_correction(spr_handle *h, int32_t enable);

/* ---- scene -------------------------------------------------------------- */
/* addVg + unifyCurveVertexOrder (ras_base.cpp:70-382, 523-569;
 * ras_cut_mask_comb_scanline.cpp:224-229).  Validates the scene, reverses
 * curves so that each runs "upward" by float bit pattern, and copies it to
 * the device.  The host arrays are not referenced after the call returns. */
int spr_set_scene(spr_handle *h, const spr_scene_view *scene);

/* The checks spr_set_scene makes, on the host only (no device needed):
 * curve types, control-point ranges, path ids in range and non-decreasing
 * along the curves, vertex path ids in range.  Returns SPR_OK,
 * SPR_ERR_INVALID_ARG (missing array) or SPR_ERR_INVALID_SCENE. */
int spr_validate_scene(const spr_scene_view *scene);

/* setInputTransform (ras_base.cpp:576-583): a row-major 4x4 matrix applied to
 * (x, y, 0, 1) followed by the reference's perspective fold (cu:36-105). */
int spr_set_transform(spr_handle *h, const float m[16]);

/* ---- gradient paints (an extension of the fill: the reference draws them
 * in its GL output shaders, ms_output_32.vert.glsl:58-103 and
 * .frag.glsl:45-51) ----------------------------------------------------------
 * A path whose fill value v satisfies 1 <= v <= 0x01000000 is painted with
 * gradient-table entry v - 1 (the reference's fill index) when a table is
 * set.  Entry layout (12 words, gradient_table_texture of rvg.cpp):
 * float tr[6] (scene -> gradient space g = (tr0 x + tr1 y + tr2,
 * tr3 x + tr4 y + tr5)), int32 first ramp texel, float (n - 1) / 1024
 * (n = ramp length), float focal[3] (fx, fy, 1 - fx^2 - fy^2 clamped at 0),
 * one unused word.  Per pixel, at its centre taken back through the reverse
 * transform (spr_set_rev_transform) and interpolated along the item's row
 * as the GL line primitive does: d = g - f, A = d.d, B = d.f,
 * c = min(A / (sqrt(B^2 + A fz) - B), 1) (0 where the denominator is not
 * above 1e-6), and the colour is the ramp sampled at c (n - 1) texels past
 * the first with linear filtering, clamped to the texel row, texels decoded
 * from sRGB first under sRGB blending.  table = NULL clears. */
int spr_set_gradients(spr_handle *h, const uint32_t *table, uint32_t n_entries, const uint32_t *ramp,
                      uint32_t n_texels);
/* ---- launch tuning (an extension) --------------------------------------------
 * Launch choices that change speed, never results: the fragment sort (0 =
 * device-wide LSD radix, 1 = one block per path segment), the curve-emission
 * order by estimated cost (0 off, 1 on), the resolve's blocks per SM (1-4)
 * and its tile: bin_width pixel columns by 64 / bin_width cell rows (the
 * band height; 64 x 1, 32 x 2, 16 x 4 or 8 x 8 cells of 2 x 2 pixels, 32
 * cells: one per lane of the warp that resolves the tile).  -1 / 0 select
 * the built-in rule (segment sort for frames of at least 1,024 paths
 * averaging at most 2,048 entries; emission order from 4,096 curves; 4
 * blocks per SM; tiles of 16 x 4 cells when the spans of the handle's last
 * sized frame covered at most 8 pixels per draw item, else 64 x 1: narrow
 * tiles cut long spans into many more resolve pairs).  Differentiable
 * frames use 64 x 1 tiles.  spr_autotune times `frames` frames of the
 * handle's scene under each choice, one choice at a time with the others at
 * their best so far, keeps the fastest (built-in rules on ties) and reports
 * it with the built-in rules' time.  Both drop a captured graph. */
typedef struct spr_tune {
    int32_t sort;
    int32_t emit_order;
    int32_t resolve_bps;
    int32_t bin_width;
    float frame_ms;   /* spr_autotune: the kept choices' mean frame time */
    float default_ms; /* spr_autotune: the built-in rules' mean frame time */
} spr_tune;

int spr_autotune(spr_handle *h, int32_t frames, void *stream, spr_tune *out);
int spr_set_tuning(spr_handle *h, const spr_tune *t);

/* setRevTransform (ras_base.cpp:595-611): screen -> scene for gradient
 * coordinates, ctx = rx[3], ry[3], rw[3], rp[3], a: rd = rx X + ry Y + rw,
 * scene = rp + (a / rd.z) rd.  Identity by default. */
int spr_set_rev_transform(spr_handle *h, const float ctx[13]);

/* ---- frame -------------------------------------------------------------- */
/* rasterize / rasterizeImpl (ras_base.cpp:1131-1195, cu:879-1453): runs the
 * whole pipeline on `stream` and leaves an RGBA8 image (row y = scene
 * y in [y, y+1), row-major, 4*width bytes per row) in device memory.  Returns
 * after the work is enqueued.  The reference reads the fragment counts back
 * twice per frame (cu:980, 1139-1157); here only the first frame after a
 * change of scene (other than one with the same path, curve and vertex
 * counts), viewport or sample count does (to size the buffers, with
 * headroom).  Later frames make no host reads: their kernels take their sizes
 * from device memory, and a frame that outgrows the buffers is rendered again
 * with larger ones when its results are first read (spr_read_image,
 * spr_image_device_ptr, spr_get_counts, spr_get_frame_stats, stage dumps).
 * Inputs changed between such a frame and that read make it
 * SPR_ERR_CAPACITY_EXCEEDED there; a bounded device wait that gave up makes it
 * SPR_ERR_TIMEOUT. */
int spr_render(spr_handle *h, void *stream);

/* Device pointer of the image written by the last spr_render. */
int spr_image_device_ptr(spr_handle *h, void **out);

/* Copies the last image to host memory (4*width*height bytes) and
 * synchronizes the stream. */
int spr_read_image(spr_handle *h, uint8_t *host_rgba, void *stream);

/* setOutputTransform / enableOutputTransform (ras_base.cpp:586-593,
 * ras_base.h:174-175): the reference's zoomed on-screen view of the image
 * (drawOutputResize, output_scale.{vert,frag}.glsl, ras_base.cpp:760-803).
 * m is row-major like spr_set_transform; a singular or non-finite inverse is
 * SPR_ERR_INVALID_ARG.  The view's pixel (x, y) is the image texel nearest to
 * inverse(m) * (x + 0.5, y + 0.5, 0, 1) after the divide by w, clamped to
 * the image (GL_NEAREST, GL_CLAMP_TO_EDGE; the coordinate is evaluated per
 * pixel, which equals GL's interpolation for affine m).  The image itself
 * (spr_read_image, spr_save_png) stays unzoomed, as saveOutputToFile's.
 * Off: the view is the image. */
int spr_set_output_transform(spr_handle *h, const float m[16]);
int spr_enable_output_transform(spr_handle *h, int32_t enable);
/* Device pointer of the view of the last image (computed on `stream` when
 * the transform is on), and its copy to host memory (synchronizes). */
int spr_output_device_ptr(spr_handle *h, void **out, void *stream);
int spr_read_output(spr_handle *h, uint8_t *host_rgba, void *stream);

/* saveOutputToFile (ras_base.cpp:1221-1277) without the exit(0): writes the
 * last image as a PNG, flipped vertically and with alpha forced to 255 like
 * the reference. */
int spr_save_png(spr_handle *h, const char *path);

/* elementNumber (ras_base.h:203). */
int spr_get_counts(spr_handle *h, spr_element_number *out);

/* enableStepTiming / stepTiming (ras_base.h:182-183, ras_base.cpp:1205-1218):
 * when enabled, spr_render records CUDA events between its stages and
 * spr_step_timing returns the per-stage milliseconds of the last frame. */
int spr_enable_step_timing(spr_handle *h, int32_t enable);
int spr_step_timing(spr_handle *h, double *ms, int32_t capacity, int32_t *n_out);
/* Graph replay (an extension: no counterpart in the reference).  When it is
 * enabled, the first spr_render after any change to the handle (scene,
 * transform, size, samples, output modes) renders normally and then captures
 * the same launch sequence, with that frame's sizes, in a CUDA graph; later
 * spr_render calls of the unchanged handle launch the graph, with no host
 * reads or synchronizations, and give the same bytes.  A reallocation of any
 * of the library's device buffers (a larger scene on another handle, a stage
 * dump, a differentiable frame) drops the graph and the next frame captures
 * again.  Off by default; frames with step timing render normally. */
int spr_set_graph_replay(spr_handle *h, int32_t enable);
/* Number of frames of this handle served by graph launches. */
int spr_graph_replays(spr_handle *h, int32_t *count);

/* Work statistics of the last spr_render. */
typedef struct spr_frame_stats {
    int32_t kernel_launches; /* CUDA kernels launched by the frame          */
    int32_t host_syncs;      /* stream synchronizations inside the frame    */
    int64_t resolve_pairs;   /* (draw item, 32-column tile) pairs resolved  */
    int64_t device_bytes;    /* device memory held by the handle            */
} spr_frame_stats;
int spr_get_frame_stats(spr_handle *h, spr_frame_stats *out);
/* Test hook of the bounded device waits (no counterpart in the reference):
 * the single-pass scans of a frame give up a look-back wait after spin_cap
 * polls (default 2^24, about a second) and the frame then fails with
 * SPR_ERR_TIMEOUT; hold_tile >= 0 makes that tile of the entry-offset scan
 * never publish its sum, so that the tiles after it wait until the limit
 * runs out (-1: none).  The handle stays usable. */
int spr_debug_set_lookback(spr_handle *h, uint32_t spin_cap, int64_t hold_tile);
/* Cap on the device memory the handle's buffers may hold, in bytes (0 = no
 * cap, the default).  The counterpart of the reference's fixed-size frame
 * arena, whose allocator throws when it is exhausted
 * (cuda_cached_allocator.h:40-115, the throw at :77-82).  A call that would
 * need more returns SPR_ERR_OUT_OF_MEMORY, as a failed device allocation
 * does; the handle stays usable (its buffers and scene are kept), and a
 * later call under a higher cap or none renders normally.  Buffers already
 * held above a lowered cap are kept until they must grow. */
int spr_set_memory_limit(spr_handle *h, int64_t bytes);
/* Name of step i of spr_step_timing (static string, NULL if out of range). */
const char *spr_step_name(int32_t i);

/* ---- stage dumps (parity testing) -------------------------------------- */
enum spr_stage {
    SPR_STAGE_TVERTEX = 0,       /* float2[n_vertices] transformed vertices          */
    SPR_STAGE_PATH_VISIBLE = 1,  /* uint8[n_paths], 1 = path passes PATH_VISIBLE     */
    SPR_STAGE_CURVE_COUNT = 2,   /* int32[n_curves] intersection entries per curve   */
    SPR_STAGE_INTERSECTION = 3,  /* int2[n_fragments] (curve id, t bits | flags)     */
    SPR_STAGE_FRAG_KEY = 4,      /* int32[n_fragments] cell key yx, raw order        */
    SPR_STAGE_FRAG_PID = 5,      /* uint32[n_fragments] path id | winding change<<30 */
    SPR_STAGE_FRAG_WN = 6,       /* int8[n_fragments] scanline winding, raw order    */
    SPR_STAGE_FRAG_MASK = 7,     /* uint32[n_fragments * samples/8] boundary masks   */
    SPR_STAGE_SORT_PERM = 8,     /* int32[n_fragments] sorted position -> raw index  */
    SPR_STAGE_SORT_KEY = 9,      /* int32[n_fragments] sorted keys                   */
    SPR_STAGE_WN_SCAN = 10,      /* int8[n_fragments] exclusive winding scan, sorted */
    SPR_STAGE_MERGED_MASK = 11,  /* uint32[merged * samples/8] final sample masks    */
    SPR_STAGE_DRAW_LIST = 12,    /* int4[merged + span] draw items                   */
    SPR_STAGE_IMAGE = 13,        /* uint8[4 * width * height]                        */
    SPR_STAGE_COUNT_ = 14
};

/* Copies stage `stage` of the last frame to host memory.  *needed receives
 * the size in bytes; nothing is copied if capacity is smaller. */
int spr_debug_dump(spr_handle *h, int32_t stage, void *host_dst, size_t capacity,
                   size_t *needed);

/* Device self-test of the resolve arithmetic: counts the float inputs in
 * [0, 1] (and slightly beyond) whose closed-form-then-corrected sRGB encode
 * differs from the threshold-table definition (expected 0). */
int spr_selftest(spr_handle *h, int64_t *srgb_encode_mismatches);

/*
 * Allocation-free exclusive scan.  No counterpart in the reference: it is an
 * extra entry point for callers that cannot allocate device memory, such as
 * plugin hosts that hand out all device memory from their own pools and
 * real-time loops that must not call cudaMalloc / cudaFree (those calls can
 * block on or synchronize the whole device).
 *
 * Writes d_offsets[i] = d_counts[0] + ... + d_counts[i-1] for i in [0, n]
 * (d_offsets holds n + 1 values; d_offsets[n] is the total), the scan that
 * turns per-curve intersection counts into entry offsets.  Both pointers are
 * device memory owned by the caller; the work is enqueued on `stream` (a
 * cudaStream_t, NULL = legacy default stream) on the current device.
 *
 * Its scratch is a fixed 64 KB array compiled into the library, which every
 * GPU that loads the library holds until the process exits.  Limit:
 * n <= 33,554,432 (16384 tiles of 2048 counts); larger n returns
 * SPR_ERR_CAPACITY_EXCEEDED and launches nothing.  Every call looks up the
 * array's device address in the current context (so a device reset or a
 * change of context between calls is followed); the first call on a device
 * also loads the array, so make that first call before any stream capture.
 * A CUDA error already pending from the caller's own work is returned as
 * SPR_ERR_CUDA, left pending, and nothing is launched.  All calls on a device
 * share the one array, so calls that overlap on the GPU (other streams, other
 * host threads) race and must be serialized by the caller.
 */
int spr_scan_offsets_noalloc(const uint32_t *d_counts, uint32_t *d_offsets, int64_t n, void *stream);

/* Human-readable text for a status code (static string). */
const char *spr_status_string(int32_t status);

/* ---- differentiable rendering (an extension: no counterpart in the reference)
 * The coverage stages are those of spr_render (bit-exact); the resolve is
 * replaced by a float composite: every sample is composited in linear RGBA
 * over opaque white in painter's order, c' = f.rgb * a + c.rgb * (1 - a),
 * c'.a = a * a + c.a * (1 - a), with the path colours f taken from
 * fill_rgba (4 floats per path) instead of path_fill_rgba, and a pixel is
 * the mean of its samples.  All pointers are device pointers.  The handle's
 * RGBA8 image is not written (batches: spr_batch_diff_render).
 */
int spr_diff_render(spr_handle *h, const float *fill_rgba, float *image, void *stream);
/* Gradients of a loss L given grad_image = dL/d(image) (4 floats per pixel):
 * grad_fill (4 per path) exactly through the composite; grad_vertex (2 per
 * input vertex, in the scene's own vertex order) and grad_affine (6 per
 * path; only with a per-path affine, else pass NULL) by edge sampling: a
 * pixel is taken as the mean over its sample rows of the row integral of
 * the composite, and every crossing of a path boundary chord with a sample
 * row contributes (c_left - c_right) dL/dI / samples to dL/dx of the
 * crossing, which moves with the chord's end points (points of the curve on
 * cell lines, or at curve ends and monotone split points) and so with the
 * control points.  Outputs are overwritten.  Right after an
 * spr_diff_render of the same inputs (nothing set or rendered in between,
 * step timing off) the backward reuses that frame's coverage stages and runs
 * the adjoint kernels only; otherwise every stage is recomputed.  256-sample
 * frames always recompute their 8 passes.  The per-sample tape grows by
 * itself (one extra readback per doubling). */
int spr_diff_backward(spr_handle *h, const float *fill_rgba, const float *grad_image, float *grad_fill,
                      float *grad_vertex, float *grad_affine, void *stream);
/* New positions of the scene's vertices (2 floats per vertex, in the scene's
 * order; host or device memory), keeping everything else of the last
 * spr_set_scene: the curves are oriented again on the device, with no host
 * synchronization (an extension, for fitting loops).  SPR_ERR_UNSUPPORTED
 * for scenes whose curves share vertices (those are oriented on the host). */
int spr_update_vertices(spr_handle *h, const float *vertex, void *stream);

/* ---- batches (an extension: no counterpart in the reference) ------------
 * Many independent scenes of uneven size rendered together: the scenes are
 * concatenated on the device, every path carries the index of its scene, and
 * one launch sequence per sample count present renders all of them, the
 * resolve taking (scene, cell row, 32-column tile) bins from one device
 * queue.  Scene i's image is RGBA8, width_i x height_i, the same bytes a
 * single-scene handle with the same settings renders for it.
 */
typedef struct spr_batch spr_batch;
typedef struct spr_batch_scene {
    spr_scene_view scene;
    int32_t width;         /* 1..4096                                        */
    int32_t height;        /* 1..4096                                        */
    int32_t samples;       /* 8, 16 or 32                                    */
    int32_t has_transform; /* 1 = transform (row-major 4x4) is applied       */
    float transform[16];
    /* optional gradient paints of this scene, as spr_set_gradients takes them
     * (12 words per entry, ramp texels in rows of 1024); n_grad = 0: none.
     * Fill values 1..n_grad use the scene's own entries. */
    const uint32_t *grad_table;
    uint32_t n_grad;
    const uint32_t *grad_ramp;
    uint32_t n_ramp;
} spr_batch_scene;
/* ms_output and srgb apply to every scene of the batch. */
int spr_batch_create(int32_t device, int32_t ms_output, int32_t srgb, spr_batch **out);
int spr_batch_destroy(spr_batch *b);
/* Validates and uploads n scenes (the arrays are copied); replaces the
 * previous set.  SPR_ERR_INVALID_SCENE / SPR_ERR_INVALID_ARG name no scene:
 * check each with spr_validate_scene to find it. */
int spr_batch_set_scenes(spr_batch *b, const spr_batch_scene *scenes, int32_t n);
int spr_batch_render(spr_batch *b, void *stream);
/* Device pointer to scene i's image (valid until the next set_scenes). */
int spr_batch_image_device_ptr(spr_batch *b, int32_t scene, void **out);
int spr_batch_read_image(spr_batch *b, int32_t scene, uint8_t *host_rgba, void *stream);
/* Totals over the scenes of the last render. */
int spr_batch_get_counts(spr_batch *b, spr_element_number *total);
int spr_batch_get_frame_stats(spr_batch *b, spr_frame_stats *out);
/* spr_set_graph_replay for every sample-count group of the batch. */
int spr_batch_set_graph_replay(spr_batch *b, int32_t enable);
/* Differentiable rendering of a batch whose scenes share one sample count
 * (else SPR_ERR_UNSUPPORTED): as spr_diff_render / spr_diff_backward /
 * spr_update_vertices, with fills, gradients and vertices of all scenes
 * concatenated in scene order and the images concatenated likewise (scene
 * i's image starts at the sum of the earlier scenes' width x height). */
int spr_batch_diff_render(spr_batch *b, const float *fill_rgba, float *image, void *stream);
int spr_batch_diff_backward(spr_batch *b, const float *fill_rgba, const float *grad_image, float *grad_fill,
                            float *grad_vertex, float *grad_affine, void *stream);
int spr_batch_update_vertices(spr_batch *b, const float *vertex, void *stream);
/* Per-step device time of the last render, summed over the sample-count
 * groups (steps as spr_step_name). */
int spr_batch_enable_step_timing(spr_batch *b, int32_t enable);
int spr_batch_step_timing(spr_batch *b, double *ms, int32_t capacity, int32_t *n_out);

/* ---- synthetic scenes ---------------------------------------------------- */
/*
 * Seeded synthetic scene generator standing in for the reference's MPVG .rvg
 * inputs, which are not available.  kind:
 *   SPR_SCENE_RANDOM  : n_paths closed paths of seg_min..seg_max segments,
 *                       40% line / 30% quadratic / 30% cubic, control points
 *                       uniform in the viewport, RGB U[0,1], alpha U[0.5,1],
 *                       fill rule 50/50 (the small plain-path scene).
 *   SPR_SCENE_MIXED   : glyph-like small paths plus large closed bands
 *                       spanning the viewport (the large plain-path scene);
 *                       n_paths = glyphs, n_large = large paths.
 *   SPR_SCENE_CUBICS  : n_paths closed paths of seg_min..seg_max cubic
 *                       segments (the differentiable-render scene).
 *   SPR_SCENE_LOCAL   : as SPR_SCENE_RANDOM, but each path's control points
 *                       are uniform in its own square box, side U[d/32, d/4]
 *                       (d = min(width, height)), placed uniformly (the
 *                       batched scenes: overdraw stays bounded as n_paths
 *                       grows).
 */
enum spr_scene_kind { SPR_SCENE_RANDOM = 0, SPR_SCENE_MIXED = 1, SPR_SCENE_CUBICS = 2, SPR_SCENE_LOCAL = 3 };

typedef struct spr_scene_spec {
    int32_t kind;
    uint64_t seed;
    int32_t width;
    int32_t height;
    int32_t n_paths;
    int32_t n_large;
    int32_t seg_min;
    int32_t seg_max;
    int32_t with_rational; /* 1 = replace 10% of quadratics with rational quadratics */
    int32_t with_affine;   /* 1 = emit per-path affine transforms (glyphs)          */
} spr_scene_spec;

typedef struct spr_scene spr_scene;

int spr_scene_generate(const spr_scene_spec *spec, spr_scene **out);
/* The view stays valid until spr_scene_free. */
int spr_scene_view_of(const spr_scene *s, spr_scene_view *view);
void spr_scene_free(spr_scene *s);

/* ---- RVG documents --------------------------------------------------------
 * RVG::load (rvg.cpp:62-776) followed by the fill conversion of
 * VGRasterizer::addVg (ras_base.cpp:138-162): the MPVG text format of the
 * reference's benchmark documents into a host scene (free with
 * spr_scene_free).  One path per element that adds vertices; M, fL, L, Q,
 * C, A (rational arcs) and Z commands; per-element dyn_affine transforms
 * applied to the vertices; solid colours truncated to 8 bits with alpha
 * times the opacity (SPR_RVG_A128: alpha quantized to 7 bits as
 * RVG::setA128).  Linear and radial paints (spread "pad") get the fill value
 * path + 1 and a gradient-table entry with its ramp (spr_scene_gradients;
 * SPR_RVG_SRGB_RAMPS: stops interpolated in linear light, for sRGB
 * rendering, as the reference does under its sRGB setting).  Relative and
 * shorthand commands return SPR_ERR_UNSUPPORTED, malformed documents
 * SPR_ERR_INVALID_SCENE, an unreadable file SPR_ERR_INVALID_ARG. */
enum spr_rvg_flags { SPR_RVG_A128 = 1, SPR_RVG_SRGB_RAMPS = 2 };
typedef struct spr_rvg_info {
    float viewport[4];        /* x0, y0, x1, y1 */
    float window[4];          /* x0, y0, x1, y1 */
    int32_t width, height;    /* the viewport's far corner as integers (RVG::width/height) */
    int32_t n_elements;       /* element lines read */
    int32_t n_gradient_paths; /* paths with a linear or radial paint */
} spr_rvg_info;

int spr_rvg_load(const char *path, int32_t flags, spr_scene **out, spr_rvg_info *info);
/* The same from a text buffer of `length` bytes. */
int spr_rvg_parse(const char *text, size_t length, int32_t flags, spr_scene **out, spr_rvg_info *info);
/* ---- the reference's scene files ---------------------------------------------
 * VGContainer::loadBinary / loadTxt (vg_container.cpp:1667-1911) for .vgb /
 * .vgt files (chosen by the name's suffix), flattened as VGRasterizer::addVg
 * does (paths, their contours, their curves in order; fill value = colour,
 * 0 when its alpha is 0, or path + 1 for gradient fills, whose table and
 * ramp come along: spr_scene_gradients; vertex path ids numbered curve by
 * curve as addVg does).  SPR_ERR_INVALID_SCENE for truncated files, indices
 * out of range, or curves whose vertex counts do not add up to the vertices.
 * spr_vg_save writes a scene in the same formats (one contour per path; no
 * per-path affines: SPR_ERR_UNSUPPORTED). */
typedef struct spr_vg_info {
    int32_t x, y, width, height; /* the container's placement and size */
    int32_t n_contours;
} spr_vg_info;

int spr_vg_load(const char *path, spr_scene **out, spr_vg_info *info);
int spr_vg_save(const spr_scene *s, int32_t width, int32_t height, const char *path);
/* A library-owned copy of a scene view (for spr_vg_save), and gradient
 * paints attached to it (12 words per table entry, ramp in rows of 1024). */
int spr_scene_from_view(const spr_scene_view *view, spr_scene **out);
int spr_scene_set_gradients(spr_scene *s, const uint32_t *table, uint32_t n_entries, const uint32_t *ramp,
                            uint32_t n_texels);

/* The scene's gradient table (12 words per entry) and ramp texels (RGBA8,
 * rows of 1024), for spr_set_gradients; zero entries for generated scenes.
 * Valid until spr_scene_free. */
int spr_scene_gradients(const spr_scene *s, const uint32_t **table, uint32_t *n_entries, const uint32_t **ramp,
                        uint32_t *n_texels);

/* ---- SVG documents -------------------------------------------------------- */
/*
 * spr_svg_load / spr_svg_parse replace SVG::load (svg_load.cpp:189-1548)
 * followed by addVg's fill conversion: the top-level <svg> elements' <g>,
 * <defs>, <path>, <polygon>, <linearGradient>, <radialGradient> and <stop>
 * elements with inherited fill, fill-rule, fill-opacity, stroke,
 * stroke-width and transform (matrix, translate, scale; rotate and skew are
 * ignored as by the reference); path data M L H V C S Q A Z in both cases
 * with the reference's reading (arcs as cubics); colours rgb(), #rgb,
 * #rrggbb.  The image is the viewBox's size (width/height when there is no
 * viewBox) with y flipped.  A stroked path is filled with its stroke colour
 * (addVg), or with SPR_SVG_STROKE_TO_FILL keeps its fill and gets an outline
 * path (spr_stroke_to_fill).  Gradient fills get the fill value path + 1 and
 * a gradient-table entry (spr_scene_gradients), which the reference's SVG
 * path never builds.  Documents with elements or values the reference cannot
 * read (rect, circle, ellipse, named colours, rgba(), T commands, style keys
 * other than stop-color / stop-opacity, objectBoundingBox gradients) return
 * SPR_ERR_UNSUPPORTED; malformed XML or numbers SPR_ERR_INVALID_SCENE; an
 * unreadable file SPR_ERR_INVALID_ARG.
 */
enum spr_svg_flags { SPR_SVG_A128 = 1, SPR_SVG_SRGB_RAMPS = 2, SPR_SVG_STROKE_TO_FILL = 4 };
typedef struct spr_svg_info {
    float view_box[4];         /* x, y, width, height */
    int32_t width, height;     /* the output size: the viewBox's, as integers */
    int32_t n_paths;           /* paths in the scene */
    int32_t n_gradient_paths;  /* paths with a gradient fill */
    int32_t n_stroked_paths;   /* paths with a stroke colour */
} spr_svg_info;

int spr_svg_load(const char *path, int32_t flags, spr_scene **out, spr_svg_info *info);
int spr_svg_parse(const char *text, size_t length, int32_t flags, spr_scene **out, spr_svg_info *info);

/* ---- stroke-to-fill ------------------------------------------------------ */
/*
 * Replaces VGContainer::strokeToOffsetCurve (vg_container.cpp:555-1353) with
 * the offset-curve approximation of SimpleBezierCurve::segApproxOffsetCurve
 * (bezier_curve.cpp:548-590): a new library-owned scene in which every input
 * path with a nonzero fill value keeps its fill path (open contours closed by
 * a line) and every path with a stroke (rgba != 0, width > 0) is followed by
 * a nonzero stroke path: per contour, butt caps, the curves offset by
 * +-width/2 (pieces within 1/32 px at their mid points, at most 128 per curve)
 * and bevel joins -- the cap and join kinds the reference's code draws.
 * `rgba` is a fill value like path_fill_rgba (RGBA8 colour, or gradient
 * entry + 1); width is in the path's own coordinates (per-path affines are
 * kept).  A contour starts at a path's first curve and wherever a curve's
 * first vertex differs from the previous curve's last.  styles holds one
 * entry per input path; a non-finite width is SPR_ERR_INVALID_ARG.  Gradient
 * tables are not copied: attach them with spr_scene_set_gradients.
 */
typedef struct spr_stroke_style {
    uint32_t rgba;
    float width;
} spr_stroke_style;

typedef struct spr_stroke_info {
    uint32_t n_fill_paths;    /* fill paths kept */
    uint32_t n_stroke_paths;  /* stroke paths added */
    uint32_t n_offset_pieces; /* offset curves emitted (caps and joins not counted) */
    int32_t max_depth;        /* deepest halving level reached (1..8) */
} spr_stroke_info;

int spr_stroke_to_fill(const spr_scene_view *in, const spr_stroke_style *styles, spr_scene **out,
                       spr_stroke_info *info);

#ifdef __cplusplus
}
#endif

#endif /* SPR_H_ */
