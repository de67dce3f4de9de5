"""Build recipe for libpbf.so, the CUDA library behind include/pbf.h.

Compiles csrc/*.cu for sm_103a only, in parallel, and links one shared
library with the CUDA runtime linked statically:

    python pbf-cuda_gb300/build.py [--force] [--ptxas-v]

Outputs: pbf-cuda_gb300/_build/*.o and pbf-cuda_gb300/lib/libpbf.so (both
git-ignored).  No cmake; nvcc from PATH or /usr/local/cuda/bin.
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
BUILD_DIR = HERE / "_build"
LIB_DIR = HERE / "lib"
LIB = LIB_DIR / "libpbf.so"
SOURCES = ["api.cu", "grid.cu", "solver.cu", "adjoint.cu", "noalloc.cu", "ssf.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    *ARCH,
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler", "-fPIC",
    # host code: round every float operation like the reference's host code
    "-Xcompiler", "-ffp-contract=off",
    "-Xcompiler", "-Wall",
]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found (needed to build libpbf.so for sm_103a)")
    return exe


def _deps() -> list[Path]:
    return (sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + sorted((HERE.parent / "include").glob("*.h")) +
            [Path(__file__)])


def _compile(src: str, ptxas_v: bool, defines=(), build_dir=None) -> tuple[str, str]:
    obj = (build_dir or BUILD_DIR) / (Path(src).stem + ".o")
    cmd = [nvcc(), *NVCC_FLAGS, *[f"-D{d}" for d in defines], "-c", str(CSRC / src), "-o", str(obj)]
    if ptxas_v:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return str(obj), r.stderr


def build(force: bool = False, ptxas_v: bool = False, verbose: bool = False, defines=(), out=None) -> Path:
    """Compile libpbf.so if it is missing or older than any source.  ``defines``
    (tuning macros) and ``out`` build a variant of the library elsewhere."""
    lib = Path(out) if out else LIB
    if lib.exists() and not force and not ptxas_v:
        t = lib.stat().st_mtime
        if all(t >= d.stat().st_mtime for d in _deps()):
            return lib
    build_dir = lib.parent / f"_build_{lib.stem}" if out else BUILD_DIR
    build_dir.mkdir(parents=True, exist_ok=True)
    lib.parent.mkdir(parents=True, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, ptxas_v, defines, build_dir), SOURCES))
    if verbose or ptxas_v:
        for _, log in results:
            if log.strip():
                print(log)
    tmp = lib.with_name(f"{lib.name}.tmp{os.getpid()}")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *[o for o, _ in results]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, ptxas_v="--ptxas-v" in sys.argv, verbose=True))
