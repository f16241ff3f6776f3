// gradients.h -- the gradient table and ramp texels of the document loaders
// (rvg_load.cpp, svg_load.cpp): one 12-word item per painted path, as the
// reference's RVG loader builds gradient_table_texture and
// gradient_ramp_texture (rvg.cpp:487-760).
#ifndef SPR_GRADIENTS_H_
#define SPR_GRADIENTS_H_

#include <cstdint>
#include <vector>

#include "spr_scene.h"

namespace spr_grad {

// One painted path's gradient item (TGradientItem, vg_container.h:59-64).
struct Item {
    float tr[6];
    int32_t p, n;
    float focal[4];
    int32_t mode;
};

struct Builder {
    std::vector<Item> items;     // one per path
    std::vector<uint32_t> ramp;  // ramp texels as built, before packing

    // A solid path's empty slot (keeps the table indexed by path).
    void solid() { items.push_back(Item{}); }
    // A linear (x0,y0 -> x1,y1) or radial (centre x0,y0, focus x1,y1,
    // radius r) paint whose gradient space maps to the scene by tr
    // (x' = tr0 x + tr1 y + tr2, y' = tr3 x + tr4 y + tr5); stops hold
    // offset, r, g, b, a (0..1) per stop.
    void paint(bool radial, const float tr[6], float x0, float y0, float x1, float y1, float r,
               std::vector<float> stops, bool srgb);
    // Packs the ramps and writes the scene's grad_table / grad_ramp.
    void finish(spr_scene &sc);
};

}  // namespace spr_grad

#endif
