"""In-tree build of libtt.so: host C++ with g++, CUDA with nvcc for sm_103a only.

Every translation unit is compiled in parallel into ``_build/`` and linked into
``trenchanttracer_gb300/libtt.so``. Host code is compiled with ``-ffp-contract=off`` so the
SBVH build and scene transforms round every operation on its own on both x86 and Arm.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libtt.so"
REPO = PKG.parent

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall", "-Wno-unused-function", "-Wno-class-memaccess"]


def _cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def _compile(src: Path, obj: Path, cuda: Path) -> Path:
    inc = ["-I" + str(REPO / "include"), "-I" + str(CSRC), "-I" + str(cuda / "include")]
    if src.suffix == ".cu":
        cmd = [str(cuda / "bin" / "nvcc"), "-O3", "-std=c++17", ARCH, "-lineinfo", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC,-ffp-contract=off", *inc, "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", *CXXFLAGS, *inc, "-c", str(src), "-o", str(obj)]
    _run(cmd)
    return obj


def sources() -> list[Path]:
    return sorted([*CSRC.glob("*.cpp"), *CSRC.glob("*.cu")])


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link libtt.so if any source is newer than the library. Concurrent callers
    (several ranks starting at once) serialise on a lock file, and only the first compiles."""
    import fcntl
    BUILD.mkdir(exist_ok=True)
    with open(BUILD / ".lock", "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        try:
            return _build_locked(force, verbose)
        finally:
            fcntl.flock(lock, fcntl.LOCK_UN)


def _build_locked(force: bool, verbose: bool) -> Path:
    cuda = _cuda_home()
    srcs = sources()
    headers = [*CSRC.glob("*.h"), *CSRC.glob("*.cuh"), *(REPO / "include").glob("*.h")]
    newest = max(p.stat().st_mtime for p in [*srcs, *headers, Path(__file__)])
    if LIB.exists() and not force and LIB.stat().st_mtime >= newest:
        return LIB
    jobs = min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = [ex.submit(_compile, s, BUILD / (s.name + ".o"), cuda) for s in srcs]
        objs = [f.result() for f in futs]
    tmp = LIB.with_suffix(".so.tmp")
    _run([str(cuda / "bin" / "nvcc"), "-shared", ARCH, "-o", str(tmp), *map(str, objs),
          "-Xcompiler", "-fopenmp", "-lgomp"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
