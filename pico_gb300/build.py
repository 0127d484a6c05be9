"""Builds libpico_gpu.so in-tree (pico_gb300/_build/) with nvcc for sm_103a.

Each translation unit compiles in parallel; an object is rebuilt when it is
older than its source or any header in csrc/ or include/.  Host code is
compiled with -ffp-contract=off because the scene builder must reproduce the
reference's float arithmetic bit for bit; device code keeps IEEE division and
square root (no fast-math) and spells its exact operations with _rn
intrinsics where the reference's operation order matters.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent
REPO = ROOT.parent
CSRC = ROOT / "csrc"
INCLUDE = REPO / "include"
BUILD = ROOT / "_build"
LIB = BUILD / "libpico_gpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["scene_build.cpp", "capi.cpp", "render.cpp", "trace.cu", "integrator.cu", "atrous.cu",
           "bsdf_eval.cu", "output.cu", "atrous_noalloc.cu", "nrc.cu", "nrc_api.cpp", "batch.cpp", "probe.cu"]


def nvcc_path() -> str:
    for cand in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        p = Path(cand) / "bin" / "nvcc"
        if cand and p.exists():
            return str(p)
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found (set CUDA_HOME)")
    return found


def _flags(src: Path) -> list[str]:
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", str(INCLUDE), "-I", str(CSRC)]
    if src.suffix == ".cu":
        return common + ARCH + ["-lineinfo", "--expt-relaxed-constexpr", "-prec-div=true",
                                "-prec-sqrt=true", "-ftz=false", "-Xptxas", "-v"]
    return common


def _newest_header() -> float:
    heads = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in heads), default=0.0)


def _compile(src: Path, obj: Path, nvcc: str) -> tuple[Path, str]:
    cmd = [nvcc, *_flags(src), "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compiles and links the library; returns its path."""
    nvcc = nvcc_path()
    BUILD.mkdir(parents=True, exist_ok=True)
    head_time = _newest_header()
    todo = []
    objs = []
    for name in SOURCES:
        src = CSRC / name
        obj = BUILD / (name.replace(".", "_") + ".o")
        objs.append(obj)
        if not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, head_time):
            todo.append((src, obj))
    logs = []
    if todo:
        with concurrent.futures.ThreadPoolExecutor(max_workers=jobs or min(8, len(todo))) as ex:
            for obj, log in ex.map(lambda so: _compile(so[0], so[1], nvcc), todo):
                logs.append((obj.name, log))
    if todo or not LIB.exists():
        cmd = [nvcc, "-shared", *ARCH, "-o", str(LIB), *map(str, objs), "-cudart", "shared"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose:
        for name, log in logs:
            print(f"== {name}\n{log}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
