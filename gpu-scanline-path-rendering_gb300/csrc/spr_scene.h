// spr_scene.h -- the library-owned host scene behind the opaque spr_scene
// handle (spr_scene_generate, spr_rvg_load): the flat scene arrays of
// spr_scene_view, owned by std::vectors.
#ifndef SPR_SCENE_H_
#define SPR_SCENE_H_

#include <cstdint>
#include <vector>

#include "../../include/spr.h"

struct spr_scene {
    std::vector<float> vertex;  // x, y per vertex
    std::vector<uint32_t> vertex_path_id;
    std::vector<uint32_t> curve_vertex_pos;
    std::vector<uint8_t> curve_type;
    std::vector<uint32_t> curve_path_id;
    std::vector<float> curve_arc_w;
    std::vector<uint8_t> fill_rule;
    std::vector<uint32_t> fill_rgba;
    std::vector<float> affine;
    bool has_affine = false;
    // gradient paints (RVG documents): 12 words per path, RGBA8 ramp texels
    std::vector<uint32_t> grad_table;
    std::vector<uint32_t> grad_ramp;

    // A curve of `type` on path `path` with control points (x, y) pairs xy.
    void add_curve(uint32_t path, int type, const float *xy, float w) {
        curve_vertex_pos.push_back((uint32_t)(vertex.size() / 2));
        curve_type.push_back((uint8_t)type);
        curve_path_id.push_back(path);
        curve_arc_w.push_back(type == SPR_CURVE_RATIONAL ? w : -1.f);
        for (int i = 0; i < (type & 7); ++i) {
            vertex.push_back(xy[2 * i]);
            vertex.push_back(xy[2 * i + 1]);
            vertex_path_id.push_back(path);
        }
    }
};

#endif
