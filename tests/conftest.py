"""Shared test setup: import paths, the `gpu` marker, built libraries."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "path-tracer_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    from pathtracer.build import build
    return build()


@pytest.fixture(scope="session")
def cornell():
    """Config 1 world: (World, full updates, oracle world)."""
    import oracle
    import pathtracer as pt
    w = pt.World.cornell_box()
    w.set_aspect_ratio(1.0)
    u = w.take_updates()
    return w, u, oracle.world_from_updates(u)
