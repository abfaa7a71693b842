"""Build the ctgpu CUDA library (sm_103a) in-tree.

Compiles every ``csrc/*.cu`` translation unit in parallel with nvcc and
links them into ``scico_gb300/_lib/libctgpu.so``.  Host code is compiled
with ``-ffp-contract=off`` so the float32 geometry tables come out the
same on x86-64 and aarch64.  Usage: ``python -m scico_gb300.build``.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
INCLUDE = REPO_DIR / "include"
OUT_DIR = PKG_DIR / "_lib"
OBJ_DIR = OUT_DIR / "obj"
LIB_NAME = "libctgpu.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off",
    "-Xptxas",
    "-warn-spills",
]


def nvcc_path() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc")
    if cand:
        return cand
    default = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(default):
        return default
    raise RuntimeError("nvcc not found: the ctgpu library needs the CUDA toolkit to build")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _compile(nvcc: str, src: Path, verbose_ptxas: bool) -> Path:
    obj = OBJ_DIR / (src.stem + ".o")
    deps = [src] + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    if obj.exists() and all(obj.stat().st_mtime >= d.stat().st_mtime for d in deps) and not verbose_ptxas:
        return obj
    cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(src), "-o", str(obj)]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
    if verbose_ptxas:
        sys.stderr.write(res.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    """Compile and link the library; return the path of the shared object."""
    nvcc = nvcc_path()
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    lib = OUT_DIR / LIB_NAME
    if force:
        for o in OBJ_DIR.glob("*.o"):
            o.unlink()
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, verbose_ptxas), srcs))
    if lib.exists() and all(lib.stat().st_mtime >= o.stat().st_mtime for o in objs):
        return lib
    tmp = OUT_DIR / (LIB_NAME + ".tmp")
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    path = build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print(path)
