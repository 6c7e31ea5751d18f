import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """libtt.so and the oracle are built in-tree once per session (a no-op when up to date)."""
    from oracle import oracle
    from trenchanttracer_gb300 import build

    build.build()
    oracle.build()


@pytest.fixture(scope="session")
def golden_dir() -> Path:
    return ROOT / "tests" / "golden"


@pytest.fixture(scope="session")
def golden_scene_files(tmp_path_factory):
    """The golden scenes written in the reference's file formats (scene JSON, OBJ, material JSON)."""
    from tests.golden import golden_scenes

    return golden_scenes.write_all(tmp_path_factory.mktemp("golden_scenes"))


def pytest_collection_modifyitems(config, items):
    """Without a CUDA device, gpu-marked tests are skipped rather than failed."""
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)
