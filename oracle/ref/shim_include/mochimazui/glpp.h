// Stand-in for the reference's GL wrapper header (not shipped in the reference
// tree).  ras_qm_mask.cu only needs these names to compile its GL sample
// query, which the host driver never calls; every call here is a no-op.
#pragma once
#define GL_RGBA8 0x8058
#define GL_TRUE 1
#define GL_COLOR_ATTACHMENT0 0x8CE0
#define GL_FRAMEBUFFER 0x8D40
#define GL_SAMPLES 0x80A9
#define GL_SAMPLE_POSITION 0x8E50
inline void glGetIntegerv(int, int *v) { *v = 0; }
inline void glGetMultisamplefv(int, int, float *v) { v[0] = v[1] = 0.f; }
namespace GLPP {
enum TextureTarget { Texture2DMultisample };
struct NamedTexture {
    NamedTexture &target(TextureTarget) { return *this; }
    NamedTexture &create() { return *this; }
    NamedTexture &storage2DMultisample(int, int, int, int, int) { return *this; }
    void destroy() {}
};
struct NamedFramebuffer {
    NamedFramebuffer &create() { return *this; }
    NamedFramebuffer &texture2D(int, const NamedTexture &, int) { return *this; }
    void bind(int) {}
    void destroy() {}
};
}  // namespace GLPP
