"""Compiles the drop-in test programs (test infrastructure)."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
HERE = Path(__file__).resolve().parent
# The reference checkout (only present where the reference is mounted; the
# tests that read it skip elsewhere): SCAFES_REFERENCE_DIR, else a
# ``reference`` directory beside this repository.
REFERENCE = Path(os.environ.get("SCAFES_REFERENCE_DIR") or ROOT.parent / "reference")


def cuda_lib_dir() -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return str(Path(nvcc).resolve().parent.parent / "lib64")


def compile_cpp(src: Path, out: Path, extra: list[str] | None = None) -> Path:
    """g++ against the drop-in headers (masterthesis_gb300/scafes) and
    libscafes_gb300.so; no reference header on the include path unless
    given in `extra`."""
    cmd = ["g++", "-std=c++14", "-O2", "-fopenmp",
           "-I", str(ROOT / "masterthesis_gb300" / "scafes"), "-I", str(ROOT / "include"),
           "-I", str(HERE)] + list(extra or []) + [
           str(src), "-o", str(out),
           "-L", str(ROOT / "masterthesis_gb300"), "-lscafes_gb300",
           "-L", cuda_lib_dir(), "-lcudart",
           f"-Wl,-rpath,{ROOT / 'masterthesis_gb300'}", f"-Wl,-rpath,{cuda_lib_dir()}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"g++ failed for {src.name}:\n{res.stderr[-4000:]}")
    return out
