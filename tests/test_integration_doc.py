"""The reference-side binding shown in INTEGRATION.md compiles against include/tt.h as written:
its C++ blocks, wrapped in one function whose parameters stand for the caller's own variables, pass
`g++ -fsyntax-only`."""
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_integration_snippets_compile_against_the_header(tmp_path):
    blocks = re.findall(r"```cpp\n(.*?)```", (ROOT / "INTEGRATION.md").read_text(), re.S)
    assert blocks
    body = "\n".join(b.replace('#include "tt.h"', "") for b in blocks)
    src = tmp_path / "binding.cpp"
    src.write_text('#include <stdexcept>\n#include <string>\n#include "tt.h"\n'
                   "void binding(const std::string &workDir, const void *d_rays, long long n, void *d_hits,\n"
                   "             void *stream, float *d_accum, float *d_accum_all, int frame, int samples,\n"
                   "             int frames) {\n" + body + "\n}\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", f"-I{ROOT / 'include'}", str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_a_c99_program_builds_a_bvh_through_the_c_abi(tmp_path):
    """include/tt.h is plain C99, and a C program linked against libtt.so can drive the host half
    of the path (scene from arrays, SBVH build, header) with no GPU."""
    prog = tmp_path / "use.c"
    prog.write_text(r'''
#include <stdio.h>
#include "tt.h"
int main(void) {
    const float v[9] = {0, 0, 0, 1, 0, 0, 0, 1, 0};
    const int32_t idx[3] = {0, 1, 2};
    tt_scene *scene = NULL;
    tt_bvh *bvh = NULL;
    tt_bvh_header h;
    if (tt_scene_create(v, 3, v, 3, idx, idx, NULL, 1, &scene) != TT_OK) return 1;
    if (tt_bvh_build(scene, 1e-5f, 1, 8, 0, &bvh) != TT_OK) return 2;
    if (tt_bvh_header_get(bvh, &h) != TT_OK) return 3;
    if (tt_bvh_build(NULL, 1e-5f, 1, 8, 0, &bvh) != TT_ERR_INVALID) return 4;
    printf("%s|%u|%u|%s\n", tt_version(), h.tri_count, h.leaf_count, tt_last_error_string());
    tt_bvh_free(bvh);
    tt_scene_free(scene);
    return 0;
}
''')
    lib_dir = ROOT / "trenchanttracer_gb300"
    exe = tmp_path / "use"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", f"-I{ROOT / 'include'}",
                        str(prog), f"-L{lib_dir}", "-ltt", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stderr)
    version, tris, leaves, err = r.stdout.strip().split("|")
    assert "sm_103a" in version and tris == "1" and int(leaves) >= 1 and err
