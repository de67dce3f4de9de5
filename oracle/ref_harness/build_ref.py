"""Build recipe of the reference harness (test infrastructure).

build_cubin():    nvcc -cubin of the reference's unmodified kernels
                  (/root/reference/fluids/Simulator.cu and the
                  Simulator_kernel.cuh it includes) plus the wrappers in
                  ref_kernels.cu, device code only, for sm_103a
                  -> oracle/_ref/ref_kernels.cubin.  Needs the reference
                  sources, so it runs where they are (this container); the
                  cubin is a GPU binary and travels to the GPU machine.
build_launcher(): the host launcher ref_launch.cu (no reference source) as a
                  shared library for the machine it runs on
                  -> oracle/_ref/libpbfref_<machine>.so.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
OUT = ROOT / "oracle" / "_ref"
CUBIN = OUT / "ref_kernels.cubin"
REFERENCE = Path("/root/reference")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def reference_present() -> bool:
    return (REFERENCE / "fluids" / "Simulator.cu").exists()


def build_cubin(force: bool = False) -> Path:
    src = HERE / "ref_kernels.cu"
    if CUBIN.exists() and not force and CUBIN.stat().st_mtime >= src.stat().st_mtime:
        return CUBIN
    OUT.mkdir(parents=True, exist_ok=True)
    tmp = CUBIN.with_suffix(f".tmp{os.getpid()}")
    cmd = [_nvcc(), "-cubin", *ARCH, "-O3", "-I", str(HERE / "stub"), "-I", str(REFERENCE / "fluids"),
           "-I", str(REFERENCE / "common" / "cuda_inc"), "-diag-suppress", "181", "-o", str(tmp), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference cubin build failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, CUBIN)
    return CUBIN


def launcher_path() -> Path:
    return OUT / f"libpbfref_{platform.machine()}.so"


def build_launcher(force: bool = False) -> Path:
    src = HERE / "ref_launch.cu"
    lib = launcher_path()
    deps = [src, ROOT / "include" / "pbf.h"]
    if lib.exists() and not force and all(lib.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return lib
    OUT.mkdir(parents=True, exist_ok=True)
    tmp = lib.with_suffix(f".tmp{os.getpid()}")
    cmd = [_nvcc(), *ARCH, "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-Xcompiler",
           "-ffp-contract=off", "-o", str(tmp), str(src), "-L", str(Path(_nvcc()).parent.parent / "lib64" / "stubs"),
           "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference launcher build failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    if reference_present():
        print(build_cubin(force=True))
    print(build_launcher(force=True))
