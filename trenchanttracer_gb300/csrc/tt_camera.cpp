// Host-side camera and frame metadata, restating the reference's Camera
// (src/core/Camera.cpp:12-44, :107-140) and WangHash (src/util/WangHash.cpp:8-15): the values
// the reference's host computes and copies to the device each frame.
#include <cmath>
#include <cstring>

#include "tt_internal.h"

namespace tt {

static const float kCameraPi = 3.14156265f;  // Camera::PI (src/core/Camera.cpp:5)

static float radians_to_degrees(float r) { return r * 180.0f / kCameraPi; }
static float degrees_to_radians(float d) { return d / 180.0f * kCameraPi; }

}  // namespace tt

using namespace tt;

extern "C" {

uint32_t tt_wang_hash(uint32_t a) {
    a = (a ^ 61u) ^ (a >> 16u);
    a = a + (a << 3u);
    a = a ^ (a >> 4u);
    a = a * 0x27d4eb2du;
    a = a ^ (a >> 15u);
    return a;
}

tt_status tt_render_meta_init(int32_t frame_number, int32_t samples, tt_render_meta *out) {
    if (!out || samples < 1) return fail(TT_ERR_INVALID, "bad argument");
    out->frame_number = frame_number;
    out->hashed_frame = tt_wang_hash((uint32_t)frame_number);
    out->samples = samples;
    out->pi = 3.14156265f;                                        // Renderer::PI (Renderer.cpp:5)
    out->two_pi = 6.2831853071795864769252867665590057683943f;    // Renderer::TWO_PI (Renderer.cpp:6)
    return TT_OK;
}

tt_status tt_camera_meta_from_scene(const tt_scene *scene, float fovx, tt_camera_meta *out) {
    if (!scene || !out) return fail(TT_ERR_INVALID, "null argument");
    const CameraConfig &c = scene->s.camera;
    if (c.width <= 0 || c.height <= 0) return fail(TT_ERR_INVALID, "scene has no camera resolution");
    // Camera::setFovx
    const float fovy = radians_to_degrees(
        std::atan(std::tan(degrees_to_radians(fovx) * 0.5f) * (float)c.height / (float)c.width) * 2.0f);
    // Camera::getCameraMeta
    const float xd = std::sin(c.yaw) * std::cos(c.pitch);
    const float yd = std::sin(c.pitch);
    const float zd = std::cos(c.yaw) * std::cos(c.pitch);
    const V3 to_cam(xd, yd, zd);
    const V3 view = to_cam * (float)(-1.0);
    const V3 eye = c.position + to_cam * c.radius;
    out->width = c.width;
    out->height = c.height;
    memcpy(out->position, &eye, 12);
    memcpy(out->view, &view, 12);
    const float up[3] = {0.f, 1.f, 0.f};
    memcpy(out->up, up, 12);
    out->fov[0] = fovx;
    out->fov[1] = fovy;
    out->aperture = c.aperture;
    out->focal = c.focal;
    return TT_OK;
}

}  // extern "C"
