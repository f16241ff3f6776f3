/*
 * spr_oracle.h -- CPU restatement of the reference's comb-scanline fill
 * pipeline.  TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and
 * the cpu_baseline / reference legs of bench.py use it as the checker.  The
 * product library (libspr) never links or calls it.
 */
#ifndef SPR_ORACLE_H_
#define SPR_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#include "../include/spr.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_config {
    int32_t width;
    int32_t height;
    int32_t samples;   /* 8, 16, 32 or 256 (8 passes of 32) */
    int32_t ms_output; /* 1 = per-sample resolve */
    int32_t srgb;      /* 1 = sRGB blending */
    int32_t threads;   /* host threads; <= 0 = all hardware threads */
    int32_t has_transform;
    float transform[16]; /* row-major 4x4, used when has_transform */
    int32_t stop_after;  /* run stages up to and including this spr_stage id (-1 = all) */
    /* gradient paints (as spr_set_gradients / spr_set_rev_transform); n_grad 0 = none */
    const uint32_t *grad_table;
    uint32_t n_grad;
    const uint32_t *grad_ramp;
    uint32_t n_ramp;
    int32_t has_rev;
    float rev[13];
} orc_config;

typedef struct orc_result orc_result;

/* Runs the pipeline on a host scene.  Returns SPR_OK or an spr_status. */
int orc_run(const spr_scene_view *scene, const orc_config *cfg, orc_result **out);
/* Pointer/size of stage `stage` (spr_stage ids); valid until orc_free. */
int orc_get(const orc_result *r, int32_t stage, const void **ptr, size_t *bytes);
int orc_counts(const orc_result *r, spr_element_number *out);
/* Wall-clock milliseconds spent in each spr_stage of the last run. */
int orc_stage_ms(const orc_result *r, double *ms, int32_t capacity);
void orc_free(orc_result *r);

/* Tables shared by the stages, exposed for table-level tests:
 *   sample positions in the 2x2-pixel cell, float2[4*samples]
 *   (index k*samples + i = sample i of pixel k, k = px.x*2 + px.y);
 *   the 256x256 half-plane mask table, uint32[65536 * samples/8];
 *   sRGB decode LUT float[256], encode thresholds float[255],
 *   encode bin base uint8[4096]. */
int orc_sample_positions(int32_t samples, float *out);
/* 256 samples per pixel render as 8 passes of 32: pass g's pixel samples
 * (float2[32], rows 8j + g of the 256-row pattern on the 32-sample rows) and
 * its half-plane table (uint32[65536 * 4]). */
int orc_pass_samples_256(int32_t pass, float *out);
int orc_pass_mask_table_256(int32_t pass, uint32_t *out);
int orc_mask_table(int32_t samples, uint32_t *out);
int orc_srgb_tables(float *decode256, float *thresholds255, uint8_t *bins4096);

/* Single-call helpers of the mask math for property tests. */
int orc_fetch_pixel_table(int32_t samples, float p0x, float p0y, float p1x, float p1y,
                          uint32_t *out_words);
int orc_vertical_mask(int32_t samples, float y, uint32_t *out_words);
/* The reference's table self-test over a res x res lattice; hist33[k] =
 * number of segments whose worst 32-bit word differs in k bits. */
int orc_fetch_table_selftest(int32_t samples, int32_t res, int64_t *hist33);
int orc_vertical_mask2(int32_t samples, float y0, float y1, uint32_t *out_words);

/* Differentiable render reference: the float composite of the draw list with
 * fill colours fill[4 * path] (linear RGBA) into image[4 * pixel], and, when
 * grad_image (dL/d(pixel), 4 per pixel) is given, the gradients of L w.r.t.
 * the fills, the input vertices (2 per vertex) and the per-path affines (6
 * per path; NULL to skip), by the same edge-sampling rule as the library. */
int orc_diff(const spr_scene_view *scene, const orc_config *cfg, const float *fill, const float *grad_image,
             double *image, double *grad_fill, double *grad_vertex, double *grad_affine);

/* Accuracy of the FP32 crossing points against FP64: for every crossing
 * entry (not piece starts) of entries[2 * n_entries] (curve id, t | flags,
 * grouped by curve id, as SPR_STAGE_INTERSECTION) of the curves whose FP32
 * transformed vertices are tvertex[2 * V] (SPR_STAGE_TVERTEX), the distance
 * along the cut line between the point the fragment stage uses (the FP32
 * curve point at the entry's t) and the exact crossing of the curve with
 * the line (FP64 root on the entry's monotone piece). */
typedef struct orc_xerr {
    double max_err_px;     /* max |along-line coordinate error|           */
    double mean_err_px;
    double max_resid_px;   /* max distance of the FP32 point from its line */
    int64_t n_crossings;
    int64_t n_over_1px;    /* crossings more than 1 px off                 */
    int64_t n_unbracketed; /* no sign change on the piece (not measured)   */
    int64_t n_mismatched;  /* entries that differ from the oracle's walk   */
    int64_t worst_entry;   /* index of the max error (-1: none)            */
} orc_xerr;
int orc_intersection_error(const spr_scene_view *scene, const float *tvertex, const int32_t *entries,
                           int64_t n_entries, int32_t width, int32_t height, int32_t threads, orc_xerr *out);

#ifdef __cplusplus
}
#endif

#endif
