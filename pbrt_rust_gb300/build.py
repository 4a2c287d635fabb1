"""Build the in-tree shared library ``_build/libpbrt_gb300.so``.

Device code is compiled for sm_103a only.  Every translation unit is built
with no floating-point contraction (``--fmad=false`` for device code,
``-ffp-contract=off`` for host code) and IEEE division/square root, so the
f32 arithmetic matches the reference crate's operation by operation.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libpbrt_gb300.so"

GENCODE = "arch=compute_103a,code=sm_103a"
CUDA_SOURCES = ["trace.cu", "reorder.cu", "render.cu", "batch.cu", "batch_trace.cu", "bvh_build.cu", "capi.cu",
                "capi_render.cu",
                "capi_noalloc.cu", "capi_batch.cu", "server.cu"]
HOST_SOURCES = ["host_scene.cpp", "image_io.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pbrt_rust_gb300")


def _cuda_home(nvcc: str) -> Path:
    return Path(nvcc).resolve().parent.parent


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build command failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    BUILD.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "pbrt_gpu.h"]
    sources = [s for s in CUDA_SOURCES + HOST_SOURCES if (CSRC / s).exists()]
    if not force and not _stale(LIB, [CSRC / s for s in sources] + headers + [Path(__file__)]):
        return LIB
    common_host = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-fno-fast-math"]
    jobs = []
    objs = []
    for s in sources:
        src = CSRC / s
        obj = BUILD / (s + ".o")
        objs.append(obj)
        if s.endswith(".cu"):
            cmd = [nvcc, "-c", str(src), "-o", str(obj), "-gencode", GENCODE, "-O3", "-lineinfo",
                   "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-std=c++17",
                   "-Xcompiler", ",".join(["-fPIC", "-ffp-contract=off", "-fno-fast-math"]),
                   "-I", str(CSRC)]
            if verbose:
                cmd += ["-Xptxas", "-v"]
        else:
            cxx = os.environ.get("CXX", "g++")
            cmd = [cxx, "-c", str(src), "-o", str(obj), *common_host, "-I", str(CSRC),
                   "-I", str(cuda / "include")]
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        futs = [ex.submit(_run, j) for j in jobs]
        for f in futs:
            f.result()
    tmp = BUILD / (LIB.name + ".tmp")
    _run([nvcc, "-shared", "-o", str(tmp), *map(str, objs), "-gencode", GENCODE,
          "-Xcompiler", "-fPIC", "-lpthread"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
