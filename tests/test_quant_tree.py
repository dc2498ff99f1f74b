"""The quantized 4-wide copy of the tree, checked on the CPU.

tests/quant_walk_check.cu (compiled here against the library's host code)
builds the reference's tree for seeded scenes, packs the quantized copy
(host_pack_quant) and checks that every decoded child box contains the exact
boxes below it, and that the quantized walk's sure-miss test plus the exact
leaf gate test exactly the triangles whose whole box path passes the
reference's slab test, with equal any-hit answers, for segments through
triangle edges, nearly axis-aligned segments and random ones; also with the
scene shifted far from the origin, where the decode rounds coarser than the
codes.  The GPU walk itself is pinned against the oracle in
tests/test_gpu_visibility.py.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "restir-vulkan_gb300" / "csrc"


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not found")
    exe = tmp_path_factory.mktemp("quant") / "quant_walk_check"
    cmd = [nvcc, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off,-fopenmp", f"-I{CSRC}",
           str(ROOT / "tests" / "quant_walk_check.cu"), str(CSRC / "host.cpp"), "-o", str(exe), "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.mark.parametrize("args", [("20000", "8000", "0", "7"), ("60000", "6000", "0", "11"),
                                  ("20000", "6000", "100000", "8"), ("20000", "6000", "-3e6", "9")],
                         ids=["near-origin", "larger", "shifted-1e5", "shifted-3e6"])
def test_quantized_walk_tests_the_reference_triangles(checker, args):
    r = subprocess.run([str(checker), *args], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    fields = dict(zip(r.stdout.split()[0::2], r.stdout.split()[1::2]))
    assert fields["containment_failures"] == "0" and fields["set_mismatches"] == "0"
    assert fields["answer_mismatches"] == "0" and int(fields["fast_rays"]) > 0
