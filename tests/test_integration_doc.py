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
