"""Shared pytest setup: import paths, the `gpu` marker, built libraries."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "restir-vulkan_gb300"
for p in (str(PKG), str(ROOT / "oracle"), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def restir_lib():
    import build as pkg_build  # restir-vulkan_gb300/build.py
    pkg_build.build()
    from restir_gb300 import _lib
    return _lib.lib()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle_binding as ob
    if not ob.LIB.exists():
        ob.build(ref=False)
    return ob


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="session")
def ctx(restir_lib, cuda):
    from restir_gb300.passes import Context
    c = Context(0)
    yield c
    c.close()
