// ref_driver.cpp -- host driver around the reference's own device code,
// compiled in place from the reference tree (see build_oracle.py): the
// intersection kernels of ras_cut.h (k_make_intersection_0/1), the mask
// helpers of ras_qm_mask.h (makeTable, fetchPixelTable, fetchVerticalTable,
// fetchVerticalTable2) and the sample pattern of ras_qm_mask.cu
// (vg_sample_position).  Each "kernel launch" is a loop that sets blockIdx.x
// and calls the kernel body once per thread index.
//
// TEST INFRASTRUCTURE ONLY: the result is a cross-check of the oracle and is
// never part of the product.  Build output goes to oracle/_ref/.

#include "ref_shim.h"

RefDim3 threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0}, blockDim = {1, 1, 1}, gridDim = {1, 1, 1};

// cutil_math.h defines host fminf/fmaxf that clash with <math.h>; include it
// once here with those two names moved aside (later includes are no-ops).
#define fminf ref_cutil_fminf
#define fmaxf ref_cutil_fmaxf
#include "cutil_math.h"
#undef fminf
#undef fmaxf

#define _MOCHIMAZUI_VG_CONTAINER_H_  // vg_container.h needs glm; only CT_* are used
#include "bezier_curve_type.h"
// ras_define.h's LAUNCH expands to a <<<...>>> launch; the only use compiled
// here is the GPU table initialisation, which this file replaces with host loops.
#include "ras_define.h"
#undef LAUNCH
#define LAUNCH(kernel, N, NT, args) ((void)0)
#include "ras_cut.h"
#include "ras_qm_mask.h"
#include "ras_qm_mask.cu"  // vg_sample_position; its GL query is stubbed

using namespace Mochimazui;

extern "C" {

// Pass 0: per-curve entry counts.  visible[p] != 0 marks a visible path.
int ref_count(int n_curves, const float *tvert, const uint32_t *vpos, const uint8_t *type,
              const uint32_t *cpid, const float *arcw, int n_paths, const uint8_t *visible, int W,
              int H, int32_t *counts, float *tcut_cache, int8_t *ncut_cache) {
    std::vector<uint64_t> vis(n_paths);
    for (int p = 0; p < n_paths; ++p) vis[p] = visible[p] ? 0x0101010101010101ull : 0ull;
    std::vector<uint32_t> vpos_m(vpos, vpos + n_curves), cpid_m(cpid, cpid + n_curves);
    std::vector<uint8_t> type_m(type, type + n_curves);
    std::vector<float> arcw_m(arcw, arcw + n_curves);
    for (int i = 0; i < n_curves; ++i) {
        blockIdx.x = i;
        Rasterizer_R_Cut::k_make_intersection_0<2, 256>(
            nullptr, (float4 *)tcut_cache, (char *)ncut_cache, counts, nullptr, type_m.data(),
            vpos_m.data(), n_curves, 0, (float2 *)tvert, arcw_m.data(), cpid_m.data(), W, H, nullptr,
            vis.data());
    }
    return 0;
}

// Pass 1: entries, given the exclusive-scan offsets of the counts and the
// monotone cut cache written by ref_count.
int ref_emit(int n_curves, const float *tvert, const uint32_t *vpos, const uint8_t *type,
             const uint32_t *cpid, const float *arcw, int n_paths, const uint8_t *visible, int W, int H,
             int32_t *offsets, float *tcut_cache, int8_t *ncut_cache, int64_t n_fragments,
             int32_t *entries) {
    std::vector<uint64_t> vis(n_paths);
    for (int p = 0; p < n_paths; ++p) vis[p] = visible[p] ? 0x0101010101010101ull : 0ull;
    std::vector<uint32_t> vpos_m(vpos, vpos + n_curves), cpid_m(cpid, cpid + n_curves);
    std::vector<uint8_t> type_m(type, type + n_curves);
    std::vector<float> arcw_m(arcw, arcw + n_curves);
    for (int i = 0; i < n_curves; ++i) {
        blockIdx.x = i;
        Rasterizer_R_Cut::k_make_intersection_1<2, 256>(
            (int2 *)entries, (float4 *)tcut_cache, (char *)ncut_cache, offsets, nullptr, type_m.data(),
            vpos_m.data(), n_curves, (int)n_fragments, (float2 *)tvert, arcw_m.data(), cpid_m.data(), W,
            H, nullptr, vis.data());
    }
    return 0;
}

// makeTable over the 256x256 table: samples = 32 cell samples of the 8-spp
// pattern followed by the 128 of the 32-spp pattern.
int ref_mask_table(const float *samples160, int32_t *out8, int32_t *out32x4) {
    std::vector<float2> s(160);
    std::memcpy(s.data(), samples160, sizeof(float2) * 160);
    for (int i = 0; i < 65536; ++i) {
        blockIdx.x = i;
        QM_Mask_2x2::makeTable(out8, (int4 *)out32x4, s.data());
    }
    return 0;
}

int ref_fetch_pixel_table(int samples, const int32_t *table, float p0x, float p0y, float p1x,
                          float p1y, int32_t *out4) {
    size_t off = 0;
    int4 r;
    if (samples == 8) {
        cudaBindTexture2D(&off, QM_Mask_2x2::tex_pixel_table8, table, cudaChannelFormatDesc{}, 256, 256,
                          256 * sizeof(int));
        r = QM_Mask_2x2::fetchPixelTable<8>(make_float2(p0x, p0y), make_float2(p1x, p1y));
    } else {
        cudaBindTexture2D(&off, QM_Mask_2x2::tex_pixel_table32, (const int4 *)table,
                          cudaChannelFormatDesc{}, 256, 256, 256 * sizeof(int4));
        r = QM_Mask_2x2::fetchPixelTable<32>(make_float2(p0x, p0y), make_float2(p1x, p1y));
    }
    out4[0] = r.x;
    out4[1] = r.y;
    out4[2] = r.z;
    out4[3] = r.w;
    return 0;
}

// vg_sample_position (ras_qm_mask.cu:118-175): the pixel sample pattern.
int ref_sample_positions(int samples, float *out_xy) {
    std::vector<float2> v = QM_Mask_Sample_Position::vg_sample_position(samples);
    for (size_t i = 0; i < v.size(); ++i) {
        out_xy[2 * i] = v[i].x;
        out_xy[2 * i + 1] = v[i].y;
    }
    return (int)v.size();
}

int ref_vertical_mask(int samples, float y, int32_t *out4) {
    int4 r = samples == 8 ? QM_Mask_2x2::fetchVerticalTable<8>(y) : QM_Mask_2x2::fetchVerticalTable<32>(y);
    out4[0] = r.x;
    out4[1] = r.y;
    out4[2] = r.z;
    out4[3] = r.w;
    return 0;
}

int ref_vertical_mask2(int samples, float y0, float y1, int32_t *out4) {
    int4 r = samples == 8 ? QM_Mask_2x2::fetchVerticalTable2<8>(y0, y1)
                          : QM_Mask_2x2::fetchVerticalTable2<32>(y0, y1);
    out4[0] = r.x;
    out4[1] = r.y;
    out4[2] = r.z;
    out4[3] = r.w;
    return 0;
}

}  // extern "C"
