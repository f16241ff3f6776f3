// spr_tables.cpp -- host-built lookup tables uploaded to the device once per
// handle: the per-cell sample pattern, the 256x256 half-plane coverage table
// (QM_Mask_2x2::makeTable, ras_qm_mask.h:432-484, built here on the host so
// that every run reads identical bits) and the sRGB tables of the resolve.
// Compiled with -ffp-contract=off.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "spr_internal.h"

namespace spr {

namespace {

// Columns of the 32-sample pattern on a 96-column lattice; the rows are the
// 32 equally spaced rows of the pixel (vg_sample_position,
// ras_qm_mask.cu:95-100, 118-175).
const uint8_t kCol32[32] = {0, 50, 24, 74, 12, 62, 38, 84, 6,  54, 30, 80, 18, 68, 42, 92,
                            3, 53, 29, 77, 17, 63, 41, 89, 9,  59, 35, 83, 21, 71, 45, 93};

// Bit reversal of i on its own bit length, as a fraction of 1.
double radical_inverse(int i) {
    int x = i, r = 0, bc = 0;
    while (x) {
        r = (r << 1) | (x & 1);
        x >>= 1;
        ++bc;
    }
    return r / (float)(1 << bc);
}

void pixel_samples(int n, float *xy) {
    if (n == 32) {
        for (int i = 0; i < 32; ++i) {
            xy[2 * i] = (float)((kCol32[i] + 0.5) / 96.0);
            xy[2 * i + 1] = (float)((2 * i + 1) / 64.0);
        }
        return;
    }
    // 8 samples: row i of 8, column = bit-reversed i (own bit length)
    // (ras_qm_mask.cu:130-163); 16 and 256 samples apply the same rule to 16
    // and 256 rows.  Rows are already in ascending y.
    const double gap = 1.0 / n, hgap = gap / 2;
    for (int i = 0; i < n; ++i) {
        int col = (int)(radical_inverse(i) * n);
        xy[2 * i] = (float)(col * gap + hgap);
        xy[2 * i + 1] = (float)(i * gap + hgap);
    }
}

// Pixel samples of pass g of a 256-sample frame: rows 8j + g of the
// 256-sample pattern (j < 32), each put on the 32-sample row (2j + 1) / 64;
// the pass moves the geometry by -pass_shift_256(g) instead.
void pass_samples_256(int g, float *xy) {
    std::vector<float> all(2 * 256);
    pixel_samples(256, all.data());
    for (int j = 0; j < 32; ++j) {
        xy[2 * j] = all[2 * (8 * j + g)];
        xy[2 * j + 1] = (float)((2 * j + 1) / 64.0);
    }
}

void cell_samples_of(const float *p, int n, float *out) {
    const float ox[4] = {0, 0, 1, 1}, oy[4] = {0, 1, 0, 1};
    for (int k = 0; k < 4; ++k)
        for (int i = 0; i < n; ++i) {
            float x = p[2 * i] + ox[k], y = p[2 * i + 1] + oy[k];
            out[2 * (k * n + i)] = x * .5f;
            out[2 * (k * n + i) + 1] = y * .5f;
        }
}

// QM_Mask_2x2::makeTable (ras_qm_mask.h:432-484) over the cell samples cs
// (n per pixel).
void mask_table_of(const float *cs, int n, uint32_t *out) {
    const int words = n / 8;
    for (int i = 0; i < 65536; ++i) {
        const int y = i / 256, x = i - y * 256;
        const float xf = ((float)x + 0.5f) * (1.f / 256.f);
        const float yf = ((float)y + 0.5f) * (1.f / 256.f);
        const float rx = 2.f * (xf - 0.5f), ry = 2.f * (yf - 0.5f);
        const float lg = std::sqrt(rx * rx + ry * ry);
        const float inv = 1.f / lg;
        float nx = inv * rx, ny = inv * ry;
        float m = 1.f - lg;
        float C = (m > 0.f ? m : 0.f) * (1.f / 0.5f);
        if (nx < 0.f) {
            nx = -nx;
            ny = -ny;
            C = -C;
        }
        if (x == 37 && y == 218) {  // the reference's hand fix for one texel
            const float il = 1.0f / std::sqrt(1.f * 1.f + (-1.f) * (-1.f));
            nx = 1.f * il;
            ny = -1.f * il;
            C = 0.f;
        }
        C += 0.5f * (nx + ny);
        for (int w = 0; w < words; ++w) {
            uint32_t bits = 0;
            for (int j = 0; j < 32; ++j) {
                const float px = cs[2 * (w * 32 + j)], py = cs[2 * (w * 32 + j) + 1];
                if (nx * px + ny * py - C > 0.f) bits |= 1u << j;
            }
            out[(size_t)i * words + w] = bits;
        }
    }
}

}  // namespace

void build_cell_samples(int n, float *out) {
    std::vector<float> p(2 * n);
    pixel_samples(n, p.data());
    cell_samples_of(p.data(), n, out);
}

void build_mask_table(int n, uint32_t *out) {
    std::vector<float> cs(8 * n);
    build_cell_samples(n, cs.data());
    mask_table_of(cs.data(), n, out);
}

void build_pass_mask_table_256(int g, uint32_t *out) {
    std::vector<float> p(2 * 32), cs(8 * 32);
    pass_samples_256(g, p.data());
    cell_samples_of(p.data(), 32, cs.data());
    mask_table_of(cs.data(), 32, out);
}

float pass_shift_256(int g) { return (float)(2 * g - 7) / 512.f; }

void build_resolve_tables(ResolveTables *t) {
    auto s2l = [](double f) { return f <= 0.04045 ? f / 12.92 : std::pow((f + 0.055) / 1.055, 2.4); };
    std::memset(t, 0, sizeof(*t));
    for (int k = 0; k < 256; ++k) {
        t->srgb_dec[k] = (float)s2l(k / 255.0);
        t->lin_dec[k] = (float)k * (1.f / 255.f);
    }
    for (int k = 0; k < 255; ++k) t->threshold[k] = (float)s2l((k + 0.5) / 255.0);
    t->threshold[255] = 2.f;
    for (int b = 0; b < 4096; ++b) {
        const float lo = (float)b * (1.f / 4096.f);
        int c = 0;
        while (c < 255 && lo >= t->threshold[c]) ++c;
        t->bin[b] = (uint8_t)c;
    }
}

}  // namespace spr
