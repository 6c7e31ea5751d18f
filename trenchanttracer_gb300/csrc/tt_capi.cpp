// Host-side C ABI: error reporting, scene creation and the SBVH / bvh.cache entry points.
#include <cfloat>
#include <cstring>
#include <new>
#include <string>

#include "tt_internal.h"

namespace tt {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

tt_status fail(tt_status code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

}  // namespace tt

using namespace tt;

#define TT_GUARD_BEGIN try {
#define TT_GUARD_END                                                      \
    }                                                                     \
    catch (const std::bad_alloc &) {                                      \
        return fail(TT_ERR_OOM, "host allocation failed");                \
    }                                                                     \
    catch (const std::exception &ex) {                                    \
        return fail(TT_ERR_INVALID, std::string("exception: ") + ex.what()); \
    }

extern "C" {

const char *tt_last_error_string(void) { return g_last_error.c_str(); }

const char *tt_version(void) { return "trenchanttracer_gb300 0.1 (sm_103a)"; }

tt_status tt_scene_load_json(const char *config_path, tt_scene **out) {
    if (!config_path || !out) return fail(TT_ERR_INVALID, "null argument");
    TT_GUARD_BEGIN
    auto *s = new tt_scene();
    tt_status st = load_scene_json(config_path, s->s);
    if (st != TT_OK) {
        delete s;
        return st;
    }
    *out = s;
    return TT_OK;
    TT_GUARD_END
}

tt_status tt_scene_create(const float *vertices, int32_t num_vertices, const float *normals, int32_t num_normals,
                          const int32_t *vidx, const int32_t *nidx, const uint32_t *mat, int32_t num_triangles,
                          tt_scene **out) {
    if (!out || num_vertices < 0 || num_normals < 0 || num_triangles < 0)
        return fail(TT_ERR_INVALID, "bad argument");
    if ((num_vertices && !vertices) || (num_normals && !normals) || (num_triangles && (!vidx || !nidx)))
        return fail(TT_ERR_INVALID, "null array");
    TT_GUARD_BEGIN
    auto *s = new tt_scene();
    Scene &sc = s->s;
    sc.vertices.resize(num_vertices);
    if (num_vertices) memcpy(sc.vertices.data(), vertices, 12ull * num_vertices);
    sc.normals.resize(num_normals);
    if (num_normals) memcpy(sc.normals.data(), normals, 12ull * num_normals);
    sc.vidx.assign(vidx, vidx + 3ll * num_triangles);
    sc.nidx.assign(nidx, nidx + 3ll * num_triangles);
    if (mat) sc.mat.assign(mat, mat + num_triangles);
    else sc.mat.assign(num_triangles, 0u);
    for (int64_t i = 0; i < 3ll * num_triangles; i++) {
        if (sc.vidx[i] < 0 || sc.vidx[i] >= num_vertices || sc.nidx[i] < 0 || sc.nidx[i] >= num_normals) {
            delete s;
            return fail(TT_ERR_INVALID, "triangle index out of range");
        }
    }
    *out = s;
    return TT_OK;
    TT_GUARD_END
}

tt_status tt_scene_counts(const tt_scene *scene, int32_t counts[5]) {
    if (!scene || !counts) return fail(TT_ERR_INVALID, "null argument");
    const Scene &sc = scene->s;
    counts[0] = sc.num_tris();
    counts[1] = (int32_t)sc.vertices.size();
    counts[2] = (int32_t)sc.normals.size();
    counts[3] = (int32_t)sc.materials.size();
    counts[4] = (int32_t)sc.geoms.size();
    return TT_OK;
}

tt_status tt_scene_arrays(const tt_scene *scene, float *vertices, float *normals, int32_t *vidx, int32_t *nidx,
                          uint32_t *mat) {
    if (!scene) return fail(TT_ERR_INVALID, "null scene");
    const Scene &sc = scene->s;
    if (vertices && !sc.vertices.empty()) memcpy(vertices, sc.vertices.data(), 12 * sc.vertices.size());
    if (normals && !sc.normals.empty()) memcpy(normals, sc.normals.data(), 12 * sc.normals.size());
    if (vidx && !sc.vidx.empty()) memcpy(vidx, sc.vidx.data(), 4 * sc.vidx.size());
    if (nidx && !sc.nidx.empty()) memcpy(nidx, sc.nidx.data(), 4 * sc.nidx.size());
    if (mat && !sc.mat.empty()) memcpy(mat, sc.mat.data(), 4 * sc.mat.size());
    return TT_OK;
}

tt_status tt_scene_env(const tt_scene *scene, int32_t *width, int32_t *height, float *rgb) {
    if (!scene || !width || !height) return fail(TT_ERR_INVALID, "null argument");
    const Scene &sc = scene->s;
    *width = sc.env_w;
    *height = sc.env_h;
    if (rgb && !sc.env_rgb.empty()) memcpy(rgb, sc.env_rgb.data(), 4 * sc.env_rgb.size());
    return TT_OK;
}

static_assert(sizeof(tt_material) == sizeof(MaterialRec) && offsetof(tt_material, ior) == offsetof(MaterialRec, ior),
              "tt_material must mirror MaterialRec");
static_assert(sizeof(tt_geometry) == sizeof(GeomRec) && offsetof(tt_geometry, p2) == offsetof(GeomRec, p2),
              "tt_geometry must mirror GeomRec");

tt_status tt_scene_set_env(tt_scene *scene, int32_t width, int32_t height, const float *rgb) {
    if (!scene || width < 0 || height < 0 || ((width > 0) != (height > 0)) || (width > 0 && !rgb))
        return fail(TT_ERR_INVALID, "bad environment map");
    TT_GUARD_BEGIN
    std::vector<float> texels(rgb, rgb + 3ll * width * height);
    // radiance is finite and not negative; anything else would poison the sampling tables
    for (size_t i = 0; i < texels.size(); i++)
        if (!(texels[i] >= 0.0f && texels[i] <= FLT_MAX))
            return fail(TT_ERR_INVALID, "environment texel value " + std::to_string(i) +
                                            " is negative, infinite or NaN");
    Scene &sc = scene->s;
    sc.env_w = width;
    sc.env_h = height;
    sc.env_rgb.swap(texels);
    return TT_OK;
    TT_GUARD_END
}

tt_status tt_scene_materials(const tt_scene *scene, tt_material *out) {
    if (!scene) return fail(TT_ERR_INVALID, "null scene");
    if (out && !scene->s.materials.empty())
        memcpy(out, scene->s.materials.data(), sizeof(MaterialRec) * scene->s.materials.size());
    return TT_OK;
}

tt_status tt_scene_set_materials(tt_scene *scene, const tt_material *materials, int32_t count) {
    if (!scene || count < 0 || (count && !materials)) return fail(TT_ERR_INVALID, "bad materials");
    for (int32_t i = 0; i < count; i++)
        if (materials[i].kind < MAT_DIFF || materials[i].kind > MAT_DIELECTRIC)
            return fail(TT_ERR_INVALID, "material " + std::to_string(i) + ": unknown kind " +
                                            std::to_string(materials[i].kind));
    TT_GUARD_BEGIN
    Scene &sc = scene->s;
    sc.materials.resize(count);
    if (count) memcpy(sc.materials.data(), materials, sizeof(MaterialRec) * count);
    sc.material_names.assign(count, std::string());
    return TT_OK;
    TT_GUARD_END
}

tt_status tt_scene_geometries(const tt_scene *scene, tt_geometry *out) {
    if (!scene) return fail(TT_ERR_INVALID, "null scene");
    if (out && !scene->s.geoms.empty()) memcpy(out, scene->s.geoms.data(), sizeof(GeomRec) * scene->s.geoms.size());
    return TT_OK;
}

tt_status tt_scene_set_geometries(tt_scene *scene, const tt_geometry *geometries, int32_t count) {
    if (!scene || count < 0 || (count && !geometries)) return fail(TT_ERR_INVALID, "bad geometries");
    for (int32_t i = 0; i < count; i++)
        if (geometries[i].kind != GEOM_SPHERE && geometries[i].kind != GEOM_PLANE)
            return fail(TT_ERR_INVALID, "analytic object " + std::to_string(i) + ": unknown kind " +
                                            std::to_string(geometries[i].kind));
    TT_GUARD_BEGIN
    scene->s.geoms.resize(count);
    if (count) memcpy(scene->s.geoms.data(), geometries, sizeof(GeomRec) * count);
    return TT_OK;
    TT_GUARD_END
}

void tt_scene_free(tt_scene *scene) { delete scene; }

tt_status tt_bvh_build(const tt_scene *scene, float split_alpha, int32_t leaf_min, int32_t leaf_max,
                       int32_t threads, tt_bvh **out) {
    if (!scene || !out) return fail(TT_ERR_INVALID, "null argument");
    if (!(split_alpha >= 0.0f)) return fail(TT_ERR_INVALID, "split_alpha must be >= 0");
    TT_GUARD_BEGIN
    BuildParams p;
    p.split_alpha = split_alpha;
    p.leaf_min = leaf_min;
    p.leaf_max = leaf_max;
    p.threads = threads;
    auto *b = new tt_bvh();
    tt_status st = build_compact(scene->s, p, b->b);
    if (st != TT_OK) {
        delete b;
        return st;
    }
    *out = b;
    return TT_OK;
    TT_GUARD_END
}

tt_status tt_bvh_save(const tt_bvh *bvh, const char *path) {
    if (!bvh || !path) return fail(TT_ERR_INVALID, "null argument");
    return save_compact(bvh->b, path);
}

tt_status tt_bvh_load(const char *path, tt_bvh **out) {
    if (!path || !out) return fail(TT_ERR_INVALID, "null argument");
    TT_GUARD_BEGIN
    auto *b = new tt_bvh();
    tt_status st = load_compact(path, b->b);
    if (st != TT_OK) {
        delete b;
        return st;
    }
    *out = b;
    return TT_OK;
    TT_GUARD_END
}

tt_status tt_bvh_header_get(const tt_bvh *bvh, tt_bvh_header *out) {
    if (!bvh || !out) return fail(TT_ERR_INVALID, "null argument");
    *out = bvh->b.hdr;
    return TT_OK;
}

tt_status tt_bvh_arrays(const tt_bvh *bvh, const void **nodes, const void **vertices, const void **normals,
                        const int32_t **tri_indices, const uint32_t **mat_indices) {
    if (!bvh) return fail(TT_ERR_INVALID, "null BVH");
    const CompactBVH &b = bvh->b;
    if (nodes) *nodes = b.nodes.data();
    if (vertices) *vertices = b.vertices.data();
    if (normals) *normals = b.normals.data();
    if (tri_indices) *tri_indices = b.tri_idx.data();
    if (mat_indices) *mat_indices = b.mat_idx.data();
    return TT_OK;
}

void tt_bvh_free(tt_bvh *bvh) { delete bvh; }

}  // extern "C"
