"""The C ABI: libtt.so loads and exports every function include/*.h declares; error reporting."""
import ctypes as C
import re
from pathlib import Path

import pytest

from trenchanttracer_gb300 import BVHCompact, TTError, _lib

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> list[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(tt_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "tt_trace" in names and "tt_bvh_build" in names and len(names) >= 15


@pytest.mark.parametrize("name", declared_functions())
def test_library_exports(name):
    lib = C.CDLL(str(_lib.LIB_PATH))
    assert hasattr(lib, name), f"libtt.so does not export {name}"


def test_python_binding_covers_header():
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_version_and_error_reporting(tmp_path):
    assert b"sm_103a" in _lib.lib().tt_version()
    with pytest.raises(TTError) as e:
        BVHCompact.load(tmp_path / "missing.cache")
    assert e.value.status == 2  # TT_ERR_IO
    assert "missing.cache" in str(e.value)


def test_null_arguments_are_rejected():
    lib = _lib.lib()
    assert lib.tt_bvh_build(None, 1e-5, 1, 8, 0, None) == 1
    assert lib.tt_trace(None, None, 0, None, 1, None) == 1
    assert lib.tt_bvh_upload(None, None) == 1


STRUCTS = {"tt_camera_meta": _lib.CameraMeta, "tt_render_meta": _lib.RenderMeta, "tt_material": _lib.Material,
           "tt_geometry": _lib.Geometry, "tt_render_params": _lib.RenderParams, "tt_bvh_header": _lib.BvhHeader,
           "tt_launch_shape": _lib.LaunchShape, "tt_view": _lib.View, "tt_cache_params": _lib.CacheParams}


def test_struct_layouts_match_the_header(tmp_path):
    """Every struct of include/tt.h has the same size and field offsets in C (gcc) and in the
    Python binding."""
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{ROOT / "include" / "tt.h"}"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    import subprocess
    subprocess.run(["gcc", "-std=c11", str(src), "-o", str(exe)], check=True)
    got = dict((" ".join(l.split()[:2]), int(l.split()[2])) for l in
               subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines())
    for cname, py in STRUCTS.items():
        assert got[f"{cname} size"] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[f"{cname} {f}"] == getattr(py, f).offset, (cname, f)


_NULL_CALLS = r"""
import ctypes as C
from trenchanttracer_gb300 import _lib
lib = _lib.lib()
ints = (C.c_int32, C.c_int64, C.c_uint32, C.c_uint64, C.c_int, C.c_size_t, C.c_longlong, C.c_ulonglong)
for name, (res, args) in _lib.SIGNATURES.items():
    if name in ("tt_version", "tt_last_error_string", "tt_wang_hash", "tt_trace_host_noalloc"):
        continue  # no handle or pointer to check; n = 0 is the allocation-free warm-up call
    vals = [0 if a in ints else 0.0 if a in (C.c_float, C.c_double) else None for a in args]
    print(name, getattr(lib, name)(*vals), flush=True)
"""


def test_every_entry_point_refuses_null_handles_and_pointers():
    """Each entry point called with NULL for every pointer and handle and 0 for every number
    returns a status other than TT_OK (the free functions return nothing), without a crash. Runs
    in a child process, so a crash names the last entry point reached."""
    import os
    import subprocess
    import sys

    pr = subprocess.run([sys.executable, "-c", _NULL_CALLS], capture_output=True, text=True, timeout=300, cwd=ROOT,
                        env={**os.environ, "PYTHONPATH": str(ROOT)})
    lines = pr.stdout.splitlines()
    assert pr.returncode == 0, (lines[-1:], pr.stderr[-1000:])
    seen = {}
    for line in lines:
        name, status = line.split()
        seen[name] = status
    free_fns = {n for n, (res, _) in _lib.SIGNATURES.items() if res is None}
    for name, status in seen.items():
        if name in free_fns:
            assert status == "None", name
        elif name not in ("tt_batch_free", "tt_cache_free"):  # freeing NULL is a no-op that succeeds
            assert status != "0", f"{name} accepted NULL arguments"
    assert len(seen) == len(_lib.SIGNATURES) - 4


def test_scene_setters_refuse_unknown_kinds():
    """Material kinds are 0-6 (the reference's five and GGX, dielectric), analytic objects are
    spheres (0) and planes (3); anything else is refused before it reaches a renderer."""
    import numpy as np
    from trenchanttracer_gb300 import Scene
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    sc = Scene.from_arrays(v, v, np.array([[0, 1, 2]], np.int32))
    lib = _lib.lib()
    mats = (_lib.Material * 2)()
    mats[0].kind, mats[1].kind = 6, 7
    assert lib.tt_scene_set_materials(sc._h, mats, 1) == 0
    assert lib.tt_scene_set_materials(sc._h, mats, 2) == 1
    assert b"unknown kind 7" in lib.tt_last_error_string()
    mats[1].kind = -1
    assert lib.tt_scene_set_materials(sc._h, mats, 2) == 1
    geoms = (_lib.Geometry * 3)()
    geoms[0].kind, geoms[1].kind, geoms[2].kind = 0, 3, 1
    assert lib.tt_scene_set_geometries(sc._h, geoms, 2) == 0
    assert lib.tt_scene_set_geometries(sc._h, geoms, 3) == 1
    assert len(sc.geometries_raw()) == 2  # a refused call leaves the scene as it was


def test_environment_setter_refuses_non_finite_or_negative_texels():
    import numpy as np
    import pytest
    from trenchanttracer_gb300 import Scene, TTError
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    sc = Scene.from_arrays(v, v, np.array([[0, 1, 2]], np.int32))
    good = np.ones((4, 8, 3), np.float32)
    sc.set_env(good)
    for bad in (np.nan, np.inf, -1e-3):
        env = good.copy()
        env[2, 5, 1] = bad
        with pytest.raises(TTError) as e:
            sc.set_env(env)
        assert e.value.status == 1 and "texel value" in str(e.value)
    assert np.array_equal(sc.env(), good)  # a refused map leaves the scene's own in place


def test_a_missing_library_fails_loudly(tmp_path):
    """The package has no fallback: a copy of it without libtt.so raises on first use instead of
    computing anything another way."""
    import os
    import shutil
    import subprocess
    import sys
    pkg = tmp_path / "trenchanttracer_gb300"
    shutil.copytree(ROOT / "trenchanttracer_gb300", pkg,
                    ignore=shutil.ignore_patterns("libtt.so", "_build", "__pycache__", "*.o", "csrc"))
    assert not (pkg / "libtt.so").exists()
    code = ("import numpy as np\n"
            "from trenchanttracer_gb300 import Scene\n"
            "v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)\n"
            "Scene.from_arrays(v, v, np.array([[0, 1, 2]], np.int32))\n")
    pr = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=tmp_path,
                        env={**os.environ, "PYTHONPATH": str(tmp_path)})
    assert pr.returncode != 0
    assert "libtt.so is missing" in pr.stderr


def test_binding_argument_counts_match_the_header():
    """Each ctypes declaration takes as many arguments as the prototype in include/tt.h."""
    protos = {}
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(tt_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text, re.S):
            params = m.group(2).strip()
            protos[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    assert len(protos) >= 60
    for name, n in protos.items():
        assert len(_lib.SIGNATURES[name][1]) == n, (name, n, len(_lib.SIGNATURES[name][1]))
