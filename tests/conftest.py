"""Shared test setup: the `gpu` marker, repo on sys.path, built artefacts."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# the reference tree: $IGAOS_REFERENCE_DIR, else `reference` beside the repository
REFERENCE = os.environ.get("IGAOS_REFERENCE_DIR") or os.path.join(
    os.path.dirname(ROOT), "reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def native():
    """Builds (if stale) and loads the engine library; never falls back."""
    from igaos_gb300 import build, capi
    build.build_lib()
    return capi.lib()


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build()
    oracle.lib()
    return oracle


def reference_dir():
    return REFERENCE if os.path.isdir(REFERENCE) else None
