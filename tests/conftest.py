"""Shared fixtures.  Registers the `gpu` marker, loads the package (whose
directory name has a hyphen) under the name wave_tool_gb300, and builds the
CPU oracle."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def wt():
    import wave_tool_gb300
    return wave_tool_gb300


@pytest.fixture(scope="session")
def oracle():
    from oracle import build, oracle as O
    build.build_oracle()
    return O


@pytest.fixture(scope="session")
def gpu(wt):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    wt.lib()  # fails loudly if the CUDA library was not built
    return torch.device("cuda:0")
