// Runs the reference's own intersect() kernel (oracle/_ref/ref_intersect.cubin, built by
// oracle/build_ref.py) on the GPU: loads the cubin through the driver API into the primary
// context, uploads the compact BVH, creates texture objects with the descriptors of
// BVHCompact::createTexture (src/bvh/BVHCompact.cpp:276-317) and launches one ray per thread,
// 256 threads per block. Also times the kernel with CUDA events (the GPU baseline).
//
// Test infrastructure only: compiled into oracle/_build/libref_gpu.so, never into libtt.so.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

static std::string g_err;

#define CK(x)                                                                 \
    do {                                                                      \
        cudaError_t e_ = (x);                                                 \
        if (e_ != cudaSuccess) {                                              \
            g_err = std::string(#x) + ": " + cudaGetErrorString(e_);          \
            goto done;                                                        \
        }                                                                     \
    } while (0)
#define CKD(x)                                                                \
    do {                                                                      \
        CUresult r_ = (x);                                                    \
        if (r_ != CUDA_SUCCESS) {                                             \
            const char *s_ = nullptr;                                         \
            cuGetErrorString(r_, &s_);                                        \
            g_err = std::string(#x) + ": " + (s_ ? s_ : "?");                 \
            goto done;                                                        \
        }                                                                     \
    } while (0)

static cudaError_t make_tex(cudaTextureObject_t *tex, void *ptr, size_t bytes, bool vec4) {
    cudaResourceDesc res;
    memset(&res, 0, sizeof(res));
    res.resType = cudaResourceTypeLinear;
    res.res.linear.devPtr = ptr;
    res.res.linear.desc.f = cudaChannelFormatKindFloat;
    res.res.linear.desc.x = 32;
    res.res.linear.desc.y = vec4 ? 32 : 0;
    res.res.linear.desc.z = vec4 ? 32 : 0;
    res.res.linear.desc.w = vec4 ? 32 : 0;
    res.res.linear.sizeInBytes = bytes;
    cudaTextureDesc td;
    memset(&td, 0, sizeof(td));
    td.readMode = cudaReadModeElementType;
    td.filterMode = cudaFilterModeLinear;
    return cudaCreateTextureObject(tex, &res, &td, nullptr);
}

extern "C" {

const char *ref_gpu_error(void) { return g_err.c_str(); }

// Host arrays in, host results out. ms_out (may be NULL) receives the median kernel time over
// `reps` launches (>= 1). Returns 0 on success.
int ref_gpu_trace(const char *cubin_path, const void *nodes, uint32_t n_nodes, const void *verts, uint32_t n_verts,
                  const void *norms, const int32_t *tri_idx, const uint32_t *mat_idx, const float *rays, int64_t n,
                  int closest, int32_t *out_id, int32_t *out_mat, float *out_t, float *out_normal, int reps,
                  float *ms_out) {
    int rc = -1;
    CUmodule mod = nullptr;
    CUfunction fn = nullptr;
    void *d_nodes = nullptr, *d_verts = nullptr, *d_norms = nullptr, *d_tri = nullptr, *d_mat = nullptr;
    float *d_rays = nullptr, *d_t = nullptr, *d_normal = nullptr;
    int *d_id = nullptr, *d_matout = nullptr;
    cudaTextureObject_t tex[5] = {0, 0, 0, 0, 0};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    float times[64];
    int nrep = reps < 1 ? 1 : (reps > 64 ? 64 : reps);
    int n32 = (int)n;
    if (n <= 0 || n > 0x7fffffff) {
        g_err = "ray count out of range";
        return -1;
    }
    CK(cudaFree(0));  // create / bind the primary context
    CKD(cuModuleLoad(&mod, cubin_path));
    CKD(cuModuleGetFunction(&fn, mod, "ref_trace_kernel"));
    CK(cudaMalloc(&d_nodes, 16ull * n_nodes));
    CK(cudaMalloc(&d_verts, 16ull * n_verts));
    CK(cudaMalloc(&d_norms, 16ull * n_verts));
    CK(cudaMalloc(&d_tri, 4ull * n_verts));
    CK(cudaMalloc(&d_mat, 4ull * n_verts));
    CK(cudaMemcpy(d_nodes, nodes, 16ull * n_nodes, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_verts, verts, 16ull * n_verts, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_norms, norms, 16ull * n_verts, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_tri, tri_idx, 4ull * n_verts, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_mat, mat_idx, 4ull * n_verts, cudaMemcpyHostToDevice));
    CK(make_tex(&tex[0], d_nodes, 16ull * n_nodes, true));
    CK(make_tex(&tex[1], d_verts, 16ull * n_verts, true));
    CK(make_tex(&tex[2], d_norms, 16ull * n_verts, true));
    CK(make_tex(&tex[3], d_tri, 4ull * n_verts, false));
    CK(make_tex(&tex[4], d_mat, 4ull * n_verts, false));
    CK(cudaMalloc(&d_rays, 32ull * n));
    CK(cudaMalloc(&d_id, 4ull * n));
    CK(cudaMalloc(&d_matout, 4ull * n));
    CK(cudaMalloc(&d_t, 4ull * n));
    CK(cudaMalloc(&d_normal, 12ull * n));
    CK(cudaMemcpy(d_rays, rays, 32ull * n, cudaMemcpyHostToDevice));
    CK(cudaEventCreate(&ev[0]));
    CK(cudaEventCreate(&ev[1]));
    {
        int cl = closest;
        void *args[] = {&d_rays, &n32, &tex[0], &tex[1], &tex[2], &tex[3], &tex[4], &cl,
                        &d_id, &d_matout, &d_t, &d_normal};
        const unsigned grid = (unsigned)((n + 255) / 256);
        for (int r = 0; r < nrep; r++) {
            CK(cudaEventRecord(ev[0], 0));
            CKD(cuLaunchKernel(fn, grid, 1, 1, 256, 1, 1, 0, nullptr, args, nullptr));
            CK(cudaEventRecord(ev[1], 0));
            CK(cudaEventSynchronize(ev[1]));
            CK(cudaEventElapsedTime(&times[r], ev[0], ev[1]));
        }
    }
    CK(cudaGetLastError());
    CK(cudaMemcpy(out_id, d_id, 4ull * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(out_t, d_t, 4ull * n, cudaMemcpyDeviceToHost));
    if (out_mat) CK(cudaMemcpy(out_mat, d_matout, 4ull * n, cudaMemcpyDeviceToHost));
    if (out_normal) CK(cudaMemcpy(out_normal, d_normal, 12ull * n, cudaMemcpyDeviceToHost));
    if (ms_out) {
        for (int i = 1; i < nrep; i++)  // insertion sort for the median
            for (int j = i; j > 0 && times[j] < times[j - 1]; j--) {
                float s = times[j];
                times[j] = times[j - 1];
                times[j - 1] = s;
            }
        *ms_out = times[nrep / 2];
    }
    rc = 0;
done:
    for (auto &t : tex)
        if (t) cudaDestroyTextureObject(t);
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    for (void *p : {d_nodes, d_verts, d_norms, d_tri, d_mat, (void *)d_rays, (void *)d_id, (void *)d_matout,
                    (void *)d_t, (void *)d_normal})
        if (p) cudaFree(p);
    if (mod) cuModuleUnload(mod);
    return rc;
}

// One frame of the reference's own pathTracingKernel (oracle/_ref/ref_render.cubin) on the scene
// given as flat arrays (see ref_render_harness.cu for geo_data / mat_data). accum (W*H*3 floats)
// is the accumulation buffer: read as the kernel's starting contents, written with its result.
// The kernel launches with the reference's own shape (16x16 blocks, grid (W/16, H/16)).
// With probe_records non-null the cubin is the probe build (ref_render_probe.cu): every material
// interaction is recorded (256 bytes each); the first ones (all of them when they fit in
// probe_capacity, else probe_capacity - 1) are copied to probe_records, and *probe_count receives
// how many the frame made.
static int render_impl(const char *cubin_path, const void *nodes, uint32_t n_nodes, const void *verts, uint32_t n_verts,
                       const void *norms, const int32_t *tri_idx, const uint32_t *mat_idx, const float *geo_data,
                       const int32_t *geo_mat, int ngeo, const float *mat_data, int nmat, const float *env_rgb,
                       int env_w, int env_h, const float *cam13, int width, int height, int frame, unsigned hashed,
                       int samples, float pi, float two_pi, float *accum, float *ms_out, void *probe_records,
                       uint64_t probe_capacity, uint64_t *probe_count) {
    int rc = -1;
    void *d_probe = nullptr;
    unsigned long long *d_probe_n = nullptr;
    CUmodule mod = nullptr;
    CUfunction f_sizes = nullptr, f_scene = nullptr, f_meta = nullptr, f_pt = nullptr;
    void *d_nodes = nullptr, *d_verts = nullptr, *d_norms = nullptr, *d_tri = nullptr, *d_mat = nullptr;
    void *d_geo_data = nullptr, *d_geo_mat = nullptr, *d_geoms = nullptr, *d_mat_data = nullptr, *d_mats = nullptr;
    void *d_env = nullptr, *d_cam = nullptr, *d_structs = nullptr, *d_accum = nullptr, *d_out = nullptr;
    int *d_sizes = nullptr;
    cudaTextureObject_t tex[7] = {0, 0, 0, 0, 0, 0, 0};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int sizes[8] = {0};
    float *env4 = nullptr;
    const size_t npx = (size_t)width * height;
    int ng = ngeo, nm = nmat, ew = env_w, eh = env_h, w = width, h = height, fr = frame, sp = samples;
    unsigned hs = hashed;
    float fpi = pi, f2pi = two_pi;
    CK(cudaFree(0));
    CKD(cuModuleLoad(&mod, cubin_path));
    CKD(cuModuleGetFunction(&f_sizes, mod, "ref_struct_sizes"));
    CKD(cuModuleGetFunction(&f_scene, mod, "ref_fill_scene"));
    CKD(cuModuleGetFunction(&f_meta, mod, "ref_fill_meta"));
    CKD(cuModuleGetFunction(&f_pt, mod,
                            "_Z17pathTracingKernelP5Vec3fS0_P8HDRImageP10RenderMetaP10CameraMetaP10BVHCompactP15"
                            "GeometryCompactP15MaterialCompact"));
    CK(cudaMalloc(&d_sizes, sizeof(sizes)));
    {
        void *args[] = {&d_sizes};
        CKD(cuLaunchKernel(f_sizes, 1, 1, 1, 1, 1, 1, 0, nullptr, args, nullptr));
    }
    CK(cudaMemcpy(sizes, d_sizes, sizeof(sizes), cudaMemcpyDeviceToHost));
    for (int i = 0; i < 6; i++) {
        if (sizes[i] <= 0 || sizes[i] > 4096) {
            g_err = "unexpected reference struct size";
            goto done;
        }
    }
    if (width < 16 || height < 16) {
        g_err = "image smaller than one 16x16 block";
        goto done;
    }
    CK(cudaMalloc(&d_nodes, 16ull * n_nodes));
    CK(cudaMalloc(&d_verts, 16ull * n_verts));
    CK(cudaMalloc(&d_norms, 16ull * n_verts));
    CK(cudaMalloc(&d_tri, 4ull * n_verts));
    CK(cudaMalloc(&d_mat, 4ull * n_verts));
    CK(cudaMemcpy(d_nodes, nodes, 16ull * n_nodes, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_verts, verts, 16ull * n_verts, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_norms, norms, 16ull * n_verts, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_tri, tri_idx, 4ull * n_verts, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_mat, mat_idx, 4ull * n_verts, cudaMemcpyHostToDevice));
    CK(make_tex(&tex[0], d_nodes, 16ull * n_nodes, true));
    CK(make_tex(&tex[1], d_verts, 16ull * n_verts, true));
    CK(make_tex(&tex[2], d_norms, 16ull * n_verts, true));
    CK(make_tex(&tex[3], d_tri, 4ull * n_verts, false));
    CK(make_tex(&tex[4], d_mat, 4ull * n_verts, false));
    CK(cudaMalloc(&d_geo_data, 64ull * (ngeo > 0 ? ngeo : 1)));
    CK(cudaMalloc(&d_geo_mat, 4ull * (ngeo > 0 ? ngeo : 1)));
    CK(cudaMalloc(&d_geoms, (size_t)sizes[7] * (ngeo > 0 ? ngeo : 1)));
    if (ngeo > 0) {
        CK(cudaMemcpy(d_geo_data, geo_data, 64ull * ngeo, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d_geo_mat, geo_mat, 4ull * ngeo, cudaMemcpyHostToDevice));
    }
    CK(make_tex(&tex[5], d_geo_mat, 4ull * (ngeo > 0 ? ngeo : 1), false));
    CK(cudaMalloc(&d_mat_data, 64ull * (nmat > 0 ? nmat : 1)));
    CK(cudaMalloc(&d_mats, (size_t)sizes[6] * (nmat > 0 ? nmat : 1)));
    if (nmat > 0) CK(cudaMemcpy(d_mat_data, mat_data, 64ull * nmat, cudaMemcpyHostToDevice));
    {
        const size_t ne = (size_t)(env_w > 0 ? env_w : 1) * (env_h > 0 ? env_h : 1);
        env4 = new float[4 * ne]();
        for (size_t i = 0; env_w > 0 && i < ne; i++) {
            env4[4 * i] = env_rgb[3 * i];
            env4[4 * i + 1] = env_rgb[3 * i + 1];
            env4[4 * i + 2] = env_rgb[3 * i + 2];
        }
        CK(cudaMalloc(&d_env, 16 * ne));
        CK(cudaMemcpy(d_env, env4, 16 * ne, cudaMemcpyHostToDevice));
        CK(make_tex(&tex[6], d_env, 16 * ne, true));
    }
    // one block of device memory for the six structs, each 256-byte aligned
    CK(cudaMalloc(&d_structs, 6 * 4096));
    CK(cudaMemset(d_structs, 0, 6 * 4096));
    CK(cudaMalloc(&d_cam, 13 * sizeof(float)));
    CK(cudaMemcpy(d_cam, cam13, 13 * sizeof(float), cudaMemcpyHostToDevice));
    {
        char *base = static_cast<char *>(d_structs);
        void *p_bvh = base, *p_geo = base + 4096, *p_matc = base + 2 * 4096, *p_hdr = base + 3 * 4096;
        void *p_rm = base + 4 * 4096, *p_cm = base + 5 * 4096;
        void *sargs[] = {&p_bvh, &tex[0], &tex[1], &tex[2], &tex[3], &tex[4], &p_geo, &d_geoms, &ng,
                         &d_geo_data, &tex[5], &p_matc, &d_mats, &nm, &d_mat_data, &p_hdr, &ew, &eh, &d_env,
                         &tex[6]};
        CKD(cuLaunchKernel(f_scene, 1, 1, 1, 1, 1, 1, 0, nullptr, sargs, nullptr));
        void *margs[] = {&p_rm, &fr, &hs, &sp, &fpi, &f2pi, &p_cm, &w, &h, &d_cam};
        CKD(cuLaunchKernel(f_meta, 1, 1, 1, 1, 1, 1, 0, nullptr, margs, nullptr));
        CK(cudaMalloc(&d_accum, 12 * npx));
        CK(cudaMalloc(&d_out, 12 * npx));
        CK(cudaMemcpy(d_accum, accum, 12 * npx, cudaMemcpyHostToDevice));
        void *pargs[] = {&d_out, &d_accum, &p_hdr, &p_rm, &p_cm, &p_bvh, &p_geo, &p_matc};
        if (probe_records) {
            CUfunction f_setup = nullptr;
            CKD(cuModuleGetFunction(&f_setup, mod, "ref_probe_setup"));
            CK(cudaMalloc(&d_probe, 256ull * (probe_capacity ? probe_capacity : 1)));
            unsigned long long cap = probe_capacity ? probe_capacity : 1;
            void *qargs[] = {&d_probe, &cap};
            CKD(cuLaunchKernel(f_setup, 1, 1, 1, 1, 1, 1, 0, nullptr, qargs, nullptr));
        }
        CK(cudaEventCreate(&ev[0]));
        CK(cudaEventCreate(&ev[1]));
        CK(cudaEventRecord(ev[0], 0));
        CKD(cuLaunchKernel(f_pt, (unsigned)(width / 16), (unsigned)(height / 16), 1, 16, 16, 1, 0, nullptr, pargs,
                           nullptr));
        CK(cudaEventRecord(ev[1], 0));
        CK(cudaEventSynchronize(ev[1]));
        if (ms_out) CK(cudaEventElapsedTime(ms_out, ev[0], ev[1]));
    }
    CK(cudaGetLastError());
    CK(cudaMemcpy(accum, d_accum, 12 * npx, cudaMemcpyDeviceToHost));
    if (probe_records) {
        CUfunction f_count = nullptr;
        unsigned long long made = 0;
        CKD(cuModuleGetFunction(&f_count, mod, "ref_probe_count"));
        CK(cudaMalloc(&d_probe_n, sizeof(made)));
        void *cargs[] = {&d_probe_n};
        CKD(cuLaunchKernel(f_count, 1, 1, 1, 1, 1, 1, 0, nullptr, cargs, nullptr));
        CK(cudaMemcpy(&made, d_probe_n, sizeof(made), cudaMemcpyDeviceToHost));
        *probe_count = made;
        // past the capacity the last slot took every further record: keep the slots before it
        const uint64_t kept = made <= probe_capacity ? made : (probe_capacity ? probe_capacity - 1 : 0);
        if (kept) CK(cudaMemcpy(probe_records, d_probe, 256ull * kept, cudaMemcpyDeviceToHost));
    }
    rc = 0;
done:
    if (d_probe) cudaFree(d_probe);
    if (d_probe_n) cudaFree(d_probe_n);
    delete[] env4;
    for (auto &t : tex)
        if (t) cudaDestroyTextureObject(t);
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    for (void *p : {d_nodes, d_verts, d_norms, d_tri, d_mat, d_geo_data, d_geo_mat, d_geoms, d_mat_data, d_mats, d_env,
                    d_cam, d_structs, d_accum, d_out, (void *)d_sizes})
        if (p) cudaFree(p);
    if (mod) cuModuleUnload(mod);
    return rc;
}

int ref_gpu_render(const char *cubin_path, const void *nodes, uint32_t n_nodes, const void *verts, uint32_t n_verts,
                   const void *norms, const int32_t *tri_idx, const uint32_t *mat_idx, const float *geo_data,
                   const int32_t *geo_mat, int ngeo, const float *mat_data, int nmat, const float *env_rgb, int env_w,
                   int env_h, const float *cam13, int width, int height, int frame, unsigned hashed, int samples,
                   float pi, float two_pi, float *accum, float *ms_out) {
    return render_impl(cubin_path, nodes, n_nodes, verts, n_verts, norms, tri_idx, mat_idx, geo_data, geo_mat, ngeo,
                       mat_data, nmat, env_rgb, env_w, env_h, cam13, width, height, frame, hashed, samples, pi, two_pi,
                       accum, ms_out, nullptr, 0, nullptr);
}

int ref_gpu_render_probe(const char *cubin_path, const void *nodes, uint32_t n_nodes, const void *verts,
                         uint32_t n_verts, const void *norms, const int32_t *tri_idx, const uint32_t *mat_idx,
                         const float *geo_data, const int32_t *geo_mat, int ngeo, const float *mat_data, int nmat,
                         const float *env_rgb, int env_w, int env_h, const float *cam13, int width, int height,
                         int frame, unsigned hashed, int samples, float pi, float two_pi, float *accum,
                         void *probe_records, uint64_t probe_capacity, uint64_t *probe_count) {
    if (!probe_records || !probe_count) {
        g_err = "probe buffers required";
        return -1;
    }
    return render_impl(cubin_path, nodes, n_nodes, verts, n_verts, norms, tri_idx, mat_idx, geo_data, geo_mat, ngeo,
                       mat_data, nmat, env_rgb, env_w, env_h, cam13, width, height, frame, hashed, samples, pi, two_pi,
                       accum, nullptr, probe_records, probe_capacity, probe_count);
}

}  // extern "C"
