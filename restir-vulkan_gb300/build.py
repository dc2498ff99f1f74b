"""Builds librestir_gb300.so in-tree for sm_103a (nvcc + the host g++).

Translation units compile in parallel; the result lands next to this file.
Every unit is compiled without FMA contraction (-fmad=false for device
code, -ffp-contract=off for host code) and with IEEE division and square
root, which the bit-exact parity of the passes depends on.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "librestir_gb300.so"
BUILD = HERE / "_build"

SOURCES = ["kernels.cu", "gbuffer_kernel.cu", "capi.cu", "noalloc.cu", "gemm_tc.cu", "mlp.cu", "proposal.cu", "batch.cu", "gpu_bvh.cu", "host.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp,-O2", "-Xptxas", "-O3",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose: bool, build_dir: Path, extra: list) -> Path:
    obj = build_dir / (src + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(CSRC / src), "-o", str(obj)]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        print(res.stderr, file=sys.stderr)
    return obj


def build(force: bool = False, verbose: bool = False, out: Path | None = None, extra_flags: list | None = None) -> Path:
    """Compiles and links the library; `out` and `extra_flags` (e.g. -D tuning
    constants) build an alternative copy elsewhere."""
    out = Path(out) if out else OUT
    extra = list(extra_flags or [])
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh"))
    deps.append(HERE.parent / "include" / "restir_gb300.h")
    if not force and not extra and out.exists() and all(out.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return out
    build_dir = BUILD if out == OUT else out.parent / "_build"
    build_dir.mkdir(parents=True, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, build_dir, extra), SOURCES))
    OUT_ = out
    tmp = OUT_.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fopenmp", "-o", str(tmp), *map(str, objs), "-lcudart_static",
           "-lrt", "-lpthread", "-ldl"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, OUT_)
    return OUT_


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
