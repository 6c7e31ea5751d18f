// Internal host-side types of libtt.so. Nothing here crosses the C ABI.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "tt_vec.h"
#include "../../include/tt.h"

namespace tt {

// ---- errors ----------------------------------------------------------------------------
void set_error(const std::string &msg);
tt_status fail(tt_status code, const std::string &msg);

// ---- materials and analytic geometry ----------------------------------------------------
// Material kinds. The first five carry the reference's MaterialType values
// (include/material/Material.h:11-13); GGX and DIELECTRIC are additions of this core.
enum MaterialKind : int32_t { MAT_DIFF = 0, MAT_METAL = 1, MAT_SPEC = 2, MAT_REFR = 3, MAT_COAT = 4,
                              MAT_GGX = 5, MAT_DIELECTRIC = 6 };

// One material, flattened for the device (a plain struct; the reference stores a
// polymorphic MaterialUnion with a vtable, include/material/MaterialUnion.h).
struct MaterialRec {
    int32_t kind;
    float emission[3];
    float color[3];      // diffuseColor (Diff/Coat) or color (Metal/Spec); GGX F0
    float color2[3];     // Coat specularColor
    float roughness;     // GGX alpha parameter (roughness^2 is the alpha)
    float ior;           // Dielectric index of refraction
    float pad[4];
};
static_assert(sizeof(MaterialRec) == 64, "MaterialRec must stay 64 B");

// Analytic geometry kinds: the reference's GeometryType values (include/geometry/Geometry.h:10-12).
enum GeomKind : int32_t { GEOM_SPHERE = 0, GEOM_CUBE = 1, GEOM_MESH = 2, GEOM_PLANE = 3 };

struct GeomRec {
    int32_t kind;
    int32_t mat;
    float radius;
    float pad;
    float p0[3];  // Plane p0, Sphere position
    float p1[3];
    float p2[3];
    float pad2[3];
};
static_assert(sizeof(GeomRec) == 64, "GeomRec must stay 64 B");

// ---- scene --------------------------------------------------------------------------------
struct CameraConfig {
    int32_t width = 0, height = 0;
    V3 position;               // orbit centre (Camera.cpp:15-18)
    float yaw = 0.f;           // Camera.cpp:20-23
    float pitch = 0.3f;        // Camera.cpp:25-28
    float focal = 4.0f;        // Camera.cpp:30-33
    float aperture = 0.04f;    // Camera.cpp:35-38
    float radius = 4.0f;       // hard-coded (Camera.cpp:40)
};

struct Scene {
    // triangle soup, as core/Scene.h keeps it
    std::vector<V3> vertices;
    std::vector<V3> normals;
    std::vector<int32_t> vidx;   // 3 per triangle
    std::vector<int32_t> nidx;   // 3 per triangle
    std::vector<uint32_t> mat;   // 1 per triangle
    // materials in scene index order and their names
    std::vector<MaterialRec> materials;
    std::vector<std::string> material_names;
    // analytic Plane/Sphere objects of the JSON scene
    std::vector<GeomRec> geoms;
    // config values of the JSON scene (src/util/Config.cpp:10-19)
    std::string work_dir, hdr_file, material_file;
    int32_t samples = 1;
    bool bvh_reload = true, material_reload = true;
    CameraConfig camera;
    // environment map: linear RGB, row 0 first, as HDRLoader leaves it
    int32_t env_w = 0, env_h = 0;
    std::vector<float> env_rgb;
    // additive keys of this core
    int32_t max_depth = 10, rr_depth = 1 << 30;

    int32_t num_tris() const { return (int32_t)mat.size(); }
};

// ---- compact BVH (host) -----------------------------------------------------------------
struct I4 { int32_t x, y, z, w; };
static_assert(sizeof(I4) == 16, "I4 must be 16 B");

struct CompactBVH {
    tt_bvh_header hdr{};
    std::vector<I4> nodes;        // 4 per inner node
    std::vector<I4> vertices;     // float bits
    std::vector<I4> normals;      // float bits
    std::vector<int32_t> tri_idx;
    std::vector<uint32_t> mat_idx;
};

struct BuildParams {
    float split_alpha = 1.0e-5f;
    int32_t leaf_min = 1;
    int32_t leaf_max = 0x7FFFFFF;
    int32_t threads = 0;
};

// SBVH build straight into the compact layout.
tt_status build_compact(const Scene &scene, const BuildParams &p, CompactBVH &out);
tt_status save_compact(const CompactBVH &b, const std::string &path);
tt_status load_compact(const std::string &path, CompactBVH &out);

// JSON scene ingest.
tt_status load_scene_json(const std::string &path, Scene &out);
tt_status load_hdr(const std::string &path, int32_t &w, int32_t &h, std::vector<float> &rgb);

}  // namespace tt

struct tt_scene {
    tt::Scene s;
};
struct tt_bvh {
    tt::CompactBVH b;
};
