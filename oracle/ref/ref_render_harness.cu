// Harness around the reference's OWN path tracer (src/core/RenderKernel.cu, pathTracingKernel),
// compiled by oracle/build_ref.py into oracle/_ref/ref_render.cubin (with the ballot shim and a
// GL-free core/Renderer.h). The reference builds its device structs on the host from C++ objects;
// these small kernels write the same structs' fields on the device instead, through the
// reference's own type definitions, so the loader needs no knowledge of their layouts.
//
// Test infrastructure only: the device oracle for the compatible path tracer.
#include <src/core/RenderKernel.cu>

extern "C" __global__ void ref_struct_sizes(int *out) {
    out[0] = (int)sizeof(BVHCompact);
    out[1] = (int)sizeof(GeometryCompact);
    out[2] = (int)sizeof(MaterialCompact);
    out[3] = (int)sizeof(HDRImage);
    out[4] = (int)sizeof(RenderMeta);
    out[5] = (int)sizeof(CameraMeta);
    out[6] = (int)sizeof(MaterialUnion);
    out[7] = (int)sizeof(GeometryUnion);
}

// geo_data: 16 floats per object: kind, p0/position xyz, p1 xyz, p2 xyz, radius.
// mat_data: 16 floats per material: kind, emission xyz, colour xyz, second colour xyz.
extern "C" __global__ void ref_fill_scene(BVHCompact *bvh, cudaTextureObject_t tn, cudaTextureObject_t tv,
                                          cudaTextureObject_t tnorm, cudaTextureObject_t ttri,
                                          cudaTextureObject_t tmat, GeometryCompact *geo, GeometryUnion *geoms,
                                          int ngeo, const float *geo_data, cudaTextureObject_t tgeomat,
                                          MaterialCompact *matc, MaterialUnion *mats, int nmat,
                                          const float *mat_data, HDRImage *hdr, int env_w, int env_h, float4 *env,
                                          cudaTextureObject_t tenv) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    bvh->nodesTexture = tn;
    bvh->verticesTexture = tv;
    bvh->normalsTexture = tnorm;
    bvh->triIndicesTexture = ttri;
    bvh->matIndicesTexture = tmat;
    geo->geometries = geoms;
    geo->geometriesSize = (U32)ngeo;
    geo->matIndicesTexture = tgeomat;
    for (int i = 0; i < ngeo; i++) {
        const float *g = geo_data + 16 * i;
        const int kind = (int)g[0];
        if (kind == PLANE) {
            Plane *p = reinterpret_cast<Plane *>(geoms + i);
            p->type = PLANE;
            p->p0 = Vec3f(g[1], g[2], g[3]);
            p->p1 = Vec3f(g[4], g[5], g[6]);
            p->p2 = Vec3f(g[7], g[8], g[9]);
        } else {
            Sphere *s = reinterpret_cast<Sphere *>(geoms + i);
            s->type = SPHERE;
            s->position = Vec3f(g[1], g[2], g[3]);
            s->radius = g[10];
        }
    }
    matc->materials = mats;
    matc->materialsSize = (U32)nmat;
    for (int i = 0; i < nmat; i++) {
        const float *m = mat_data + 16 * i;
        Material *mm = reinterpret_cast<Material *>(mats + i);
        mm->index = (U32)i;
        mm->type = (MaterialType)(int)m[0];
        mm->emission = Vec3f(m[1], m[2], m[3]);
        const Vec3f c1(m[4], m[5], m[6]), c2(m[7], m[8], m[9]);
        switch (mm->type) {
            case DIFF: reinterpret_cast<Diff *>(mm)->diffuseColor = c1; break;
            case METAL: reinterpret_cast<Metal *>(mm)->color = c1; break;
            case SPEC: reinterpret_cast<Spec *>(mm)->color = c1; break;
            case COAT:
                reinterpret_cast<Coat *>(mm)->diffuseColor = c1;
                reinterpret_cast<Coat *>(mm)->specularColor = c2;
                break;
            default: break;
        }
    }
    hdr->width = env_w;
    hdr->height = env_h;
    hdr->hdrEnv = env;
    hdr->hdrTexture = tenv;
}

// cam: resolution via w/h, then 13 floats: position, view, up, fov xy, aperture, focal.
extern "C" __global__ void ref_fill_meta(RenderMeta *rm, int frame, unsigned hashed, int samples, float pi,
                                         float two_pi, CameraMeta *cm, int w, int h, const float *cam) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    rm->frameNumber = frame;
    rm->hashedFrame = hashed;
    rm->SAMPLES = samples;
    rm->PI = pi;
    rm->TWO_PI = two_pi;
    cm->resolution = Vec2i(w, h);
    cm->position = Vec3f(cam[0], cam[1], cam[2]);
    cm->view = Vec3f(cam[3], cam[4], cam[5]);
    cm->up = Vec3f(cam[6], cam[7], cam[8]);
    cm->fov = Vec2f(cam[9], cam[10]);
    cm->apertureRadius = cam[11];
    cm->focalDistance = cam[12];
}
