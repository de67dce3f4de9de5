"""Build recipe of the reference harness (test infrastructure).

The reference checkout is taken from the PBF_REFERENCE environment variable
(default: /root/reference, where this build's container mounts it).

build_cubin():    nvcc -cubin of the reference's unmodified kernels
                  (<reference>/fluids/Simulator.cu and the
                  Simulator_kernel.cuh it includes) plus the wrappers in
                  ref_kernels.cu, device code only, for sm_103a
                  -> oracle/_ref/ref_kernels.cubin.  Needs the reference
                  sources, so it runs where they are (this container); the
                  cubin is a GPU binary and travels to the GPU machine.
build_launcher(): the host launcher ref_launch.cu (no reference source) as a
                  shared library for the machine it runs on
                  -> oracle/_ref/libpbfref_<machine>.so.
build_ssf_ref():  the reference's SSF shaders (fluids/shader/SSF*.glsl), made
                  C++ by a few syntax rewrites (glsl_as_cpp) into
                  oracle/_ref/ssf_shaders.inc, compiled with the CPU harness
                  ssf_ref.cpp -> oracle/_ref/libssfref_<machine>.so.  Needs the
                  reference sources, so it runs where they are.
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
# the reference checkout (read-only; nothing is written there)
REFERENCE = Path(os.environ.get("PBF_REFERENCE", "/root/reference"))
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


# ---- the reference's SSF shaders on the CPU -------------------------------------------

SHADER_DIR = REFERENCE / "fluids" / "shader"
# namespace in the generated file -> shader source (fluids/SSFRenderer.cpp:89-93)
SHADERS = {
    "ref_depth_v": "SSFget_depth.v.glsl",
    "ref_depth_f": "SSFget_depth.f.glsl",
    "ref_thick_v": "SSFget_thick.v.glsl",
    "ref_thick_f": "SSFget_thick.f.glsl",
    "ref_smooth_f": "SSFsmooth_depth.f.glsl",
    "ref_normal_f": "SSFrestore_normal.f.glsl",
    "ref_shading_f": "SSFshading.f.glsl",
}
SHADERS_INC = OUT / "ssf_shaders.inc"


def ssf_shaders_present() -> bool:
    return all((SHADER_DIR / f).exists() for f in SHADERS.values())


def glsl_as_cpp(text: str) -> str:
    """The rewrites that make a GLSL shader C++ (ssf_glsl.hpp supplies the
    types, built-ins and functions): drop the #version / #extension lines,
    make float literals float, turn the read-only swizzles .xyz / .rgb / .xy
    into calls and .r into .x.  The in / out / uniform / layout qualifiers and
    discard are macros around the include; main is renamed there."""
    import re

    lines = [ln for ln in text.splitlines() if not re.match(r"^\s*#\s*(version|extension)\b", ln)]
    out = "\n".join(lines)
    out = re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)(?![\w.])", r"\1f", out)
    out = re.sub(r"\.(xyz|rgb)\b", ".xyz()", out)
    out = re.sub(r"\.xy\b", ".xy()", out)
    out = re.sub(r"\.r\b", ".x", out)
    return out


def generate_ssf_shaders() -> Path:
    """oracle/_ref/ssf_shaders.inc: each shader in its own namespace."""
    OUT.mkdir(parents=True, exist_ok=True)
    parts = ["// generated by oracle/ref_harness/build_ref.py from fluids/shader/SSF*.glsl", "#define uniform",
             "#define in", "#define out", "#define layout(...)", "#define discard (glsl::gl_discarded = true)",
             "#define main shader_main"]
    for ns, f in SHADERS.items():
        parts += [f"namespace {ns} {{", "using namespace glsl;", f"#line 1 \"{f}\"",
                  glsl_as_cpp((SHADER_DIR / f).read_text()), f"}}  // namespace {ns}"]
    parts += ["#undef main", "#undef discard", "#undef layout", "#undef out", "#undef in", "#undef uniform", ""]
    tmp = SHADERS_INC.with_suffix(f".tmp{os.getpid()}")
    tmp.write_text("\n".join(parts))
    os.replace(tmp, SHADERS_INC)
    return SHADERS_INC


def ssf_ref_path() -> Path:
    return OUT / f"libssfref_{platform.machine()}.so"


def build_ssf_ref(force: bool = False) -> Path:
    """g++ of ssf_ref.cpp (ours) with the generated shader file -> oracle/_ref/libssfref_<machine>.so."""
    lib = ssf_ref_path()
    src = HERE / "ssf_ref.cpp"
    deps = [src, HERE / "ssf_glsl.hpp", Path(__file__), ROOT / "include" / "pbf_ssf.h"]
    deps += [SHADER_DIR / f for f in SHADERS.values()]
    if lib.exists() and not force and all(lib.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return lib
    generate_ssf_shaders()
    tmp = lib.with_suffix(f".tmp{os.getpid()}")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w", "-I", str(OUT), "-I", str(HERE),
           "-o", str(tmp), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference shader harness build failed:\n{r.stderr[-6000:]}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    if reference_present():
        print(build_cubin(force=True))
    if ssf_shaders_present():
        print(build_ssf_ref(force=True))
    print(build_launcher(force=True))
