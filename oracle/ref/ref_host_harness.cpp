// C entry points around the reference's OWN host code, compiled from the reference sources by
// oracle/build_ref.py into oracle/_ref/libttref_host.so (never committed, never shipped in
// libtt.so). They let the tests run the reference's scene loader, SBVH builder and a
// host-compiled intersect() on the same inputs as this project's code.
//
// Test infrastructure only.
#include <omp.h>

#include <cstdio>
#include <cstring>
#include <exception>
#include <string>

#include <bvh/BVH.h>
#include <bvh/BVHCompact.h>
#include <bvh/SAHHelper.h>
#include <core/Camera.h>
#include <core/Group.h>
#include <core/Scene.h>
#include <geometry/Plane.h>
#include <geometry/Sphere.h>
#include <material/Coat.h>
#include <material/Diff.h>
#include <material/Metal.h>
#include <material/Spec.h>
#include <hdr/HDRImage.h>
#include <loader/HDRLoader.h>
#include <loader/SceneLoader.h>
#include <util/Config.h>
#include <util/WangHash.h>

#include "ref_host_compat.h"
#include <geometry/IntersectKernel.cuh>

extern "C" {

// Config -> SceneLoader::load -> BVH(scene, SAHHelper{leaf prefs}, alpha) -> BVHCompact::save,
// the sequence of src/main.cpp:34-75.
int ref_build_json(const char *config_path, const char *cache_path, float split_alpha, int leaf_min,
                   int leaf_max) {
    try {
        Config config(config_path);
        SceneLoader loader(&config);
        Scene *scene = loader.load();
        SAHHelper sah;
        sah.setLeafPreferences(leaf_min, leaf_max);
        BVH bvh(scene, sah, split_alpha);
        BVHCompact *compact = bvh.createHolder();
        compact->save(cache_path);
        delete compact;
        delete scene;
        return 0;
    } catch (const std::exception &e) {
        fprintf(stderr, "ref_build_json: %s\n", e.what());
        return -1;
    }
}

// Scene arrays as the reference's loader leaves them: counts[0..2] = triangles, vertices,
// normals; then the caller passes buffers of those sizes (NULL to query counts only).
int ref_scene_arrays(const char *config_path, int *counts, float *vertices, float *normals, int *vidx, int *nidx,
                     unsigned *mat) {
    try {
        Config config(config_path);
        SceneLoader loader(&config);
        Scene *scene = loader.load();
        counts[0] = scene->getTrianglesNum();
        counts[1] = scene->getVerticesNum();
        counts[2] = scene->getNormalNum();
        if (vertices) memcpy(vertices, scene->getVertexPtr(), 12ull * counts[1]);
        if (normals) memcpy(normals, scene->getNormalPtr(), 12ull * counts[2]);
        if (vidx) memcpy(vidx, scene->getTrianglePtr(), 12ull * counts[0]);
        if (nidx) memcpy(nidx, scene->getNormalIndexPtr(), 12ull * counts[0]);
        if (mat) memcpy(mat, scene->getMatIndexPtr(), 4ull * counts[0]);
        delete scene;
        return 0;
    } catch (const std::exception &e) {
        fprintf(stderr, "ref_scene_arrays: %s\n", e.what());
        return -1;
    }
}

// Camera(config) + setFovx(45) + getCameraMeta(), as src/main.cpp:37-38 and Renderer::display
// use them. out = position xyz, view xyz, up xyz, fov xy, aperture, focal (13 floats).
int ref_camera_meta(const char *config_path, float fovx, float *out) {
    try {
        Config config(config_path);
        Camera camera(&config);
        camera.setFovx(fovx);
        CameraMeta m = camera.getCameraMeta();
        const float v[13] = {m.position.x, m.position.y, m.position.z, m.view.x, m.view.y, m.view.z,
                             m.up.x, m.up.y, m.up.z, m.fov.x, m.fov.y, m.apertureRadius, m.focalDistance};
        memcpy(out, v, sizeof(v));
        return 0;
    } catch (const std::exception &e) {
        fprintf(stderr, "ref_camera_meta: %s\n", e.what());
        return -1;
    }
}

unsigned ref_wang_hash(unsigned a) { return WangHash::encode(a); }

// The materials and analytic objects the reference's loader leaves in the Scene, flattened.
// counts[0..1] = materials, analytic objects; pass NULL buffers to query the counts. Per material
// 10 floats: type, emission xyz, the first colour xyz (Diff / Coat: diffuseColor, Metal / Spec:
// color), the second xyz (Coat: specularColor), zeros where a kind has none. Per analytic object
// 13 floats: type, material index, radius (Sphere), 0, then p0 (Sphere: position), p1, p2.
int ref_scene_materials(const char *config_path, int *counts, float *mats, float *geoms) {
    try {
        Config config(config_path);
        SceneLoader loader(&config);
        Scene *scene = loader.load();
        counts[0] = scene->getMaterialNum();
        counts[1] = scene->getGeometryNum();
        for (int i = 0; mats && i < counts[0]; i++) {
            const Material *m = scene->getMaterial(i);
            float *o = mats + 10 * i;
            memset(o, 0, 10 * sizeof(float));
            o[0] = (float)m->type;
            o[1] = m->emission.x, o[2] = m->emission.y, o[3] = m->emission.z;
            Vec3f a(0, 0, 0), b(0, 0, 0);
            if (m->type == DIFF) a = ((const Diff *)m)->diffuseColor;
            if (m->type == METAL) a = ((const Metal *)m)->color;
            if (m->type == SPEC) a = ((const Spec *)m)->color;
            if (m->type == COAT) a = ((const Coat *)m)->diffuseColor, b = ((const Coat *)m)->specularColor;
            o[4] = a.x, o[5] = a.y, o[6] = a.z, o[7] = b.x, o[8] = b.y, o[9] = b.z;
        }
        for (int i = 0; geoms && i < counts[1]; i++) {
            const Group *g = scene->getGeometry(i);
            const Geometry *geo = g->getGeometry();
            float *o = geoms + 13 * i;
            memset(o, 0, 13 * sizeof(float));
            o[0] = (float)geo->type;
            o[1] = (float)g->getMaterial()->index;
            if (geo->type == SPHERE) {
                const Sphere *sp = (const Sphere *)geo;
                o[2] = sp->radius;
                o[4] = sp->position.x, o[5] = sp->position.y, o[6] = sp->position.z;
            } else if (geo->type == PLANE) {
                const Plane *pl = (const Plane *)geo;
                const Vec3f *p[3] = {&pl->p0, &pl->p1, &pl->p2};
                for (int k = 0; k < 3; k++) o[4 + 3 * k] = p[k]->x, o[5 + 3 * k] = p[k]->y, o[6 + 3 * k] = p[k]->z;
            }
        }
        delete scene;
        return 0;
    } catch (const std::exception &e) {
        fprintf(stderr, "ref_scene_materials: %s\n", e.what());
        return -1;
    }
}

// The reference's intersect() compiled for the host (ballot -> this lane only; video min/max ->
// integer min/max), over n rays of 8 floats under OpenMP. Loads the BVH from bvh.cache with
// the reference's own reader (BVHCompact(FILE*)).
int ref_intersect_host(const char *cache_path, const float *rays, long long n, int closest, int *idx, int *mat,
                       float *t, float *normal, int threads) {
    FILE *f = fopen(cache_path, "rb");
    if (!f) return -1;
    try {
        BVHCompact bvh(f);
        if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 4096)
        for (long long i = 0; i < n; i++) {
            const float *r = rays + 8 * i;
            Ray ray(Vec3f(r[0], r[1], r[2]), Vec3f(r[3], r[4], r[5]), r[6], r[7]);
            Hit h = intersect(ray, &bvh, closest != 0);
            idx[i] = h.index;
            t[i] = h.distance;
            if (mat) mat[i] = h.index != -1 ? h.matIndex : -1;
            if (normal) {
                normal[3 * i + 0] = h.normal.x;
                normal[3 * i + 1] = h.normal.y;
                normal[3 * i + 2] = h.normal.z;
            }
        }
        return 0;
    } catch (const std::exception &e) {
        fprintf(stderr, "ref_intersect_host: %s\n", e.what());
        return -1;
    }
}

// HDRLoader::load (src/loader/HDRLoader.cpp:5-62): the decoded picture as the reference keeps it,
// rows in file order, 3 floats per texel (read back from the HDRImage's float4 array, which the
// cudart stub holds in host memory). Returns -1 when the loader throws or the picture exceeds cap
// floats.
int ref_load_hdr(const char *path, int *w, int *h, float *rgb, long long cap) {
    try {
        HDRLoader loader;
        HDRImage *img = loader.load(path);
        const long long n = (long long)img->width * img->height;
        *w = img->width;
        *h = img->height;
        if (3 * n > cap) {
            delete img;
            return -1;
        }
        const float *src = reinterpret_cast<const float *>(img->hdrEnv);
        for (long long i = 0; i < n; i++)
            for (int c = 0; c < 3; c++) rgb[3 * i + c] = src[4 * i + c];
        delete img;
        return 0;
    } catch (const std::exception &e) {
        fprintf(stderr, "ref_load_hdr: %s\n", e.what());
        return -1;
    }
}

}  // extern "C"
