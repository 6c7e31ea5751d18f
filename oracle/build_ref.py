"""Builds the reference's own code into oracle/_ref/ (git-ignored), to check the oracle and the
CUDA path against.

Outputs:
  oracle/_ref/libttref_host.so   the reference's scene loader, SBVH builder, BVHCompact writer,
                                 Camera and intersect() compiled for the host (g++, OpenMP), with
                                 a cudart stub standing in for device memory
  oracle/_ref/ref_intersect.cubin the reference's device intersect() inside a one-ray-per-thread
                                 harness, compiled for sm_103a
  oracle/_ref/ref_render*.cubin  the reference's pathTracingKernel: as written (ref_render), with its
                                 material interactions recorded (ref_render_probe), and with
                                 intersect()'s warp vote taken per lane (ref_render_lane_vote)

The reference sources are compiled where they lie under the reference checkout. Exactly two
headers are shadowed by patched copies written to a temporary directory (deleted afterwards):
  geometry/IntersectKernel.cuh  host build: the video min/max asm becomes integer min/max and the
                                warp ballot tests this lane only; device build: the legacy
                                `vote.ballot.b32` (rejected by ptxas for sm_70+) becomes
                                `activemask` + `vote.sync.ballot.b32` on that mask
  core/Renderer.h               the GL/GLUT includes and the Renderer class dropped (RenderMeta kept)
The .cubin is device code only, so it is also usable on an Arm GPU host where the reference
checkout is absent; libttref_host.so is x86 host code and is rebuilt wherever sources exist.

Usage: python oracle/build_ref.py [--reference PATH]
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
DEFAULT_REF = Path(os.environ.get("TT_REFERENCE_DIR", "/root/reference"))

HOST_SOURCES = [
    "src/bvh/AABB.cpp", "src/bvh/BVH.cpp", "src/bvh/BVHCompact.cpp", "src/bvh/BVHNode.cpp",
    "src/bvh/InnerNode.cpp", "src/bvh/LeafNode.cpp", "src/bvh/SAHHelper.cpp",
    "src/util/Sort.cpp", "src/util/Config.cpp", "src/util/WangHash.cpp",
    "src/core/Scene.cpp", "src/core/Object.cpp", "src/core/Group.cpp", "src/core/Camera.cpp",
    "src/geometry/Transform.cpp", "src/geometry/Mesh.cpp", "src/geometry/Geometry.cpp",
    "src/geometry/Plane.cpp", "src/geometry/Sphere.cpp", "src/geometry/GeometryCompact.cpp",
    "src/material/Material.cpp", "src/material/MaterialPool.cpp", "src/material/MaterialCompact.cpp",
    "src/material/Diff.cpp", "src/material/Metal.cpp", "src/material/Spec.cpp", "src/material/Refr.cpp",
    "src/material/Coat.cpp", "src/loader/SceneLoader.cpp", "src/loader/OBJLoader.cpp",
    "src/loader/MaterialLoader.cpp", "src/loader/HDRLoader.cpp", "src/hdr/HDRImage.cpp",
]

VMIN = {
    'asm("vmin.s32.s32.s32.min %0, %1, %2, %3;" : "=r"(v) : "r"(a), "r"(b), "r"(c));':
        "v = std::min(std::min(a, b), c);",
    'asm("vmin.s32.s32.s32.max %0, %1, %2, %3;" : "=r"(v) : "r"(a), "r"(b), "r"(c));':
        "v = std::max(std::min(a, b), c);",
    'asm("vmax.s32.s32.s32.min %0, %1, %2, %3;" : "=r"(v) : "r"(a), "r"(b), "r"(c));':
        "v = std::min(std::max(a, b), c);",
    'asm("vmax.s32.s32.s32.max %0, %1, %2, %3;" : "=r"(v) : "r"(a), "r"(b), "r"(c));':
        "v = std::max(std::max(a, b), c);",
}
# core/Renderer.h without its GL/GLUT/GL-interop includes and the Renderer class: the scene,
# HDR and kernel headers only need RenderMeta (include/core/Renderer.h:24-31) from it.
RENDERER_STUB = """#ifndef TRENCHANTTRACER_RENDERER_H
#define TRENCHANTTRACER_RENDERER_H
#include <cuda_runtime.h>
#include <core/Scene.h>
#include <core/Camera.h>
#include <math/LinearMath.h>
#include <util/Config.h>
#include <util/WangHash.h>
#include <bvh/BVHCompact.h>
#include <material/MaterialCompact.h>
#include <geometry/GeometryCompact.h>
struct RenderMeta {
    int frameNumber;
    unsigned int hashedFrame;
    int SAMPLES;
    float PI;
    float TWO_PI;
};
class HDRImage;
class Renderer {
public:
    Vec3f *accumulatedBuffer;
    Vec3f *outputBuffer;
    CameraMeta *cameraMetaDevice;
    RenderMeta renderMeta;
    RenderMeta *renderMetaDevice;
    Config *config;
    BVHCompact *bvhCompact;
    GeometryCompact *geometryCompact;
    MaterialCompact *materialCompact;
    HDRImage *hdrEnv;
    void render();
};
#endif
"""
BALLOT_LINE = '"vote.ballot.b32    %0,p;       \\n"'
BALLOT_SHIM = '"activemask.b32 %0;\\n vote.sync.ballot.b32 %0, p, %0;\\n"'


def _patch(text: str, old: str, new: str) -> str:
    if text.count(old) != 1:
        raise SystemExit(f"build_ref: pattern not found exactly once in IntersectKernel.cuh: {old!r}")
    return text.replace(old, new)


def _host_kernel_header(src: str) -> str:
    for old, new in VMIN.items():
        src = _patch(src, old, new)
    start = src.index('asm("{\\n"')
    end = src.index(': "r"(leafAddr));', start) + len(': "r"(leafAddr));')
    src = src[:start] + "mask = (leafAddr >= 0) ? 1u : 0u;" + src[end:]
    return "#include <algorithm>\n" + src


def _gpu_kernel_header(src: str) -> str:
    return _patch(src, BALLOT_LINE, BALLOT_SHIM)


def _gpu_lane_vote_header(src: str) -> str:
    """The device kernel with its warp vote made per lane: a lane stops looking for leaves when it
    has found one itself, not when every lane of its warp has (the per-ray algorithm)."""
    start = src.index('asm("{\\n"')
    end = src.index(': "r"(leafAddr));', start) + len(': "r"(leafAddr));')
    return src[:start] + "mask = (leafAddr >= 0) ? 1u : 0u;" + src[end:]


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise SystemExit("build_ref failed:\n" + " ".join(cmd) + "\n" + proc.stdout[-6000:])


def build(ref: Path = DEFAULT_REF, quiet: bool = True) -> bool:
    """Returns False (and builds nothing) when the reference checkout is absent."""
    if not (ref / "include" / "geometry" / "IntersectKernel.cuh").exists():
        return False
    OUT.mkdir(exist_ok=True)
    cuda = Path(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc").resolve().parent.parent
    kernel = (ref / "include" / "geometry" / "IntersectKernel.cuh").read_text()
    with tempfile.TemporaryDirectory(prefix="ttref_") as tmp:
        tmp = Path(tmp)
        host_inc = tmp / "host" / "geometry"
        gpu_inc = tmp / "gpu" / "geometry"
        lane_inc = tmp / "lane" / "geometry"
        host_inc.mkdir(parents=True)
        gpu_inc.mkdir(parents=True)
        lane_inc.mkdir(parents=True)
        (host_inc / "IntersectKernel.cuh").write_text(_host_kernel_header(kernel))
        (gpu_inc / "IntersectKernel.cuh").write_text(_gpu_kernel_header(kernel))
        (lane_inc / "IntersectKernel.cuh").write_text(_gpu_lane_vote_header(kernel))
        for side in ("host", "gpu", "lane"):
            (tmp / side / "core").mkdir()
            (tmp / side / "core" / "Renderer.h").write_text(RENDERER_STUB)

        lib = OUT / "libttref_host.so"
        srcs = [str(ref / s) for s in HOST_SOURCES]
        objs = []
        # compile in parallel, one object per source
        procs = []
        objdir = tmp / "obj"
        objdir.mkdir()
        common = ["g++", "-O2", "-std=c++14", "-fPIC", "-fopenmp", "-w",
                  "-I" + str(tmp / "host"), "-I" + str(HERE / "ref"), "-I" + str(ref / "include"),
                  "-I" + str(ref / "lib" / "include"), "-I" + str(cuda / "include")]
        for s in srcs + [str(HERE / "ref" / "cudart_stub.cpp"), str(HERE / "ref" / "ref_host_harness.cpp")]:
            o = objdir / (Path(s).name + ".o")
            objs.append(str(o))
            procs.append((subprocess.Popen(common + ["-c", s, "-o", str(o)], stdout=subprocess.PIPE,
                                           stderr=subprocess.STDOUT, text=True), s))
        for p, s in procs:
            out, _ = p.communicate()
            if p.returncode != 0:
                raise SystemExit(f"build_ref: {s} failed:\n{out[-4000:]}")
        # -Bsymbolic: the reference's CUDA runtime calls bind to the host stub linked in here even
        # when the process already holds the real libcudart (torch loads it into the global scope)
        _run(["g++", "-shared", "-fopenmp", "-Wl,-Bsymbolic", "-o", str(lib), *objs])

        cubin = OUT / "ref_intersect.cubin"
        _run([str(cuda / "bin" / "nvcc"), "-cubin", "-gencode=arch=compute_103a,code=sm_103a", "-w",
              "-I" + str(tmp / "gpu"), "-I" + str(ref / "include"), "-I" + str(ref / "lib" / "include"),
              str(HERE / "ref" / "ref_gpu_harness.cu"), "-o", str(cubin)])
        # the reference's pathTracingKernel (RenderKernel.cu) with struct-filling helpers
        _run([str(cuda / "bin" / "nvcc"), "-cubin", "-gencode=arch=compute_103a,code=sm_103a", "-w",
              "-I" + str(tmp / "gpu"), "-I" + str(ref / "include"), "-I" + str(ref / "lib" / "include"),
              "-I" + str(ref), str(HERE / "ref" / "ref_render_harness.cu"), "-o", str(OUT / "ref_render.cubin")])
        # the same kernel with intersect()'s warp vote made per lane (nothing else changed)
        _run([str(cuda / "bin" / "nvcc"), "-cubin", "-gencode=arch=compute_103a,code=sm_103a", "-w",
              "-I" + str(tmp / "lane"), "-I" + str(ref / "include"), "-I" + str(ref / "lib" / "include"),
              "-I" + str(ref), str(HERE / "ref" / "ref_render_harness.cu"), "-o",
              str(OUT / "ref_render_lane_vote.cubin")])
        # the same kernel with every material interaction recorded (ref_render_probe.cu)
        _run([str(cuda / "bin" / "nvcc"), "-cubin", "-gencode=arch=compute_103a,code=sm_103a", "-w",
              "-I" + str(tmp / "gpu"), "-I" + str(ref / "include"), "-I" + str(ref / "lib" / "include"),
              "-I" + str(ref), str(HERE / "ref" / "ref_render_probe.cu"), "-o",
              str(OUT / "ref_render_probe.cubin")])
    if not quiet:
        print(f"built {OUT}/libttref_host.so and ref_intersect.cubin", file=sys.stderr)
    return True


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", type=Path, default=DEFAULT_REF)
    a = ap.parse_args()
    if not build(a.reference, quiet=False):
        print("reference checkout not found; oracle/_ref keeps its prebuilt files", file=sys.stderr)
