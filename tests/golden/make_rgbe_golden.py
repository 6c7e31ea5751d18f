"""Writes tests/golden/rgbe_golden.json: sha256 of the reference HDRLoader's decoded floats for
each picture of tests/golden/rgbe_files.py (needs oracle/_ref/libttref_host.so, built from the
reference sources by oracle/build_ref.py).

Usage: python tests/golden/make_rgbe_golden.py
"""
from __future__ import annotations

import hashlib
import json
import sys
import tempfile
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import refhost  # noqa: E402
from tests.golden.rgbe_files import write_all  # noqa: E402


def main() -> None:
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for name, path in write_all(Path(d)).items():
            img = refhost.load_hdr(str(path))
            out[name] = {"shape": list(img.shape), "sha256": hashlib.sha256(img.tobytes()).hexdigest(),
                         "sum": float(img.astype("float64").sum())}
    (Path(__file__).parent / "rgbe_golden.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
