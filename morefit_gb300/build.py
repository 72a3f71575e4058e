"""Builds the native library of the MoreFit GB300 backend in-tree.

``build_library()`` compiles ``morefit_gb300/csrc`` into
``morefit_gb300/_build/libmorefit_cuda.so`` with nvcc for sm_103a
(``-gencode arch=compute_103a,code=sm_103a``), translation units in
parallel, CUDA runtime linked statically and NVRTC dynamically from the
toolkit. The build is skipped when the library is newer than every source.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
INCLUDE = PKG.parent / "include"
LIB = OUT / "libmorefit_cuda.so"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    p = CUDA_HOME / "bin" / "nvcc"
    return str(p) if p.exists() else "nvcc"


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cpp")) + list(CSRC.glob("*.cu")))


def _deps() -> list[Path]:
    return _sources() + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _compile(src: Path) -> Path:
    obj = OUT / (src.stem + ".o")
    cmd = [_nvcc(), "-std=c++17", "-O3", GENCODE, "-lineinfo", "-Xcompiler", "-fPIC,-O3",
           "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cu":
        cmd[5:5] = ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    if src.suffix == ".cu":
        (OUT / (src.stem + ".ptxas.txt")).write_text(r.stderr)
    return obj


def build_library(force: bool = False) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    if LIB.exists() and not force:
        newest = max(p.stat().st_mtime for p in _deps())
        if LIB.stat().st_mtime >= newest:
            return LIB
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(_compile, _sources()))
    tmp = OUT / (LIB.name + f".tmp{os.getpid()}")
    cmd = [_nvcc(), "-shared", GENCODE, "-o", str(tmp), *map(str, objs),
           "-L", str(CUDA_HOME / "lib64"), "-lnvrtc", "-cudart", "static",
           "-Xlinker", f"-rpath,{CUDA_HOME / 'lib64'}", "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(force=True))
