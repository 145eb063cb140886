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


def read_device_form(path) -> dict:
    """The named FP64 arrays of a Problem::dumpDeviceForm file."""
    import numpy as np
    b = Path(path).read_bytes()
    out, i = {}, 0
    while i < len(b):
        name = b[i:i + 16].split(b"\0")[0].decode()
        n = int(np.frombuffer(b[i + 16:i + 24], dtype=np.int64)[0])
        i += 24
        out[name] = np.frombuffer(b[i:i + 8 * n], dtype=np.float64)
        i += 8 * n
    return out


def tissue_args(golden: dict, workdir: Path) -> list[str]:
    """Command-line options of run_problem / extract_reference for a tissue
    golden case: the grid, the time axis, the example's constants and (MRI)
    its known fields written to a raw FP64 file."""
    import numpy as np
    n = [int(v) for v in golden["n"]]
    last = [float(v) for v in golden["last"]]
    args = [f"--nNodes={n[0]}x{n[1]}x{n[2]}", f"--coordNodeLast={last[0]!r}x{last[1]!r}x{last[2]!r}",
            f"--tau={float(golden['tau'])!r}", f"--nTimesteps={int(golden['nsteps'])}",
            f"--endtime={float(golden['t_end'])!r}",
            "--params=" + ",".join(repr(float(v)) for v in golden["params"])]
    if "fields" in golden:
        path = Path(workdir) / "fields.bin"
        np.concatenate([golden["fields"].ravel(), golden["surface"].ravel()]).tofile(path)
        args.append(f"--fields={path}")
    return args
