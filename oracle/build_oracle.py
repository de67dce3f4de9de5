"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/pbf_oracle.c and oracle/ssf_oracle.c twice each (float port +
FP64 oracle) into one shared library, oracle/_build/liboracle.so, with gcc and OpenMP.  Portable C: the same
recipe builds on x86_64 and aarch64 hosts.

    python oracle/build_oracle.py
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "pbf_oracle.c"
SSF_SRC = HERE / "ssf_oracle.c"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "liboracle.so"
CFLAGS = ["-O2", "-fPIC", "-std=gnu11", "-fopenmp", "-ffp-contract=off", "-Wall", "-Wno-unknown-pragmas"]


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the oracle library if it is missing or older than its sources."""
    deps = [SRC, SSF_SRC, HERE.parent / "include" / "pbf.h", HERE.parent / "include" / "pbf_ssf.h", Path(__file__)]
    if LIB.exists() and not force and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    objs = []
    for src in (SRC, SSF_SRC):
        for tag, defs in (("f32", []), ("f64", ["-DORACLE_F64"])):
            obj = OUT_DIR / f"{src.stem}_{tag}.o"
            cmd = ["gcc", *CFLAGS, *defs, "-c", str(src), "-o", str(obj)]
            if verbose:
                print(" ".join(cmd))
            subprocess.run(cmd, check=True)
            objs.append(str(obj))
    tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
    subprocess.run(["gcc", "-shared", "-fopenmp", "-o", str(tmp), *objs, "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


SAN_FLAGS = ["-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined"]


def build_sanitized(out_dir: Path) -> Path:
    """The same library built with AddressSanitizer and UndefinedBehaviorSanitizer
    into out_dir (tests/test_oracle_sanitized.py), for a process started with
    the sanitizer runtimes preloaded."""
    out_dir = Path(out_dir)
    out_dir.mkdir(parents=True, exist_ok=True)
    flags = [f for f in CFLAGS if not f.startswith("-O")] + SAN_FLAGS
    objs = []
    for src in (SRC, SSF_SRC):
        for tag, defs in (("f32", []), ("f64", ["-DORACLE_F64"])):
            obj = out_dir / f"{src.stem}_{tag}.o"
            subprocess.run(["gcc", *flags, *defs, "-c", str(src), "-o", str(obj)], check=True)
            objs.append(str(obj))
    lib = out_dir / "liboracle.so"
    subprocess.run(["gcc", "-shared", "-fopenmp", "-fsanitize=address,undefined", "-o", str(lib), *objs, "-lm"],
                   check=True)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
