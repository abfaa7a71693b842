"""Build the C/OpenMP restatement (oracle/ctref.c) into oracle/_build/:
libctref.so (float32, the reference's precision) and libctref64.so (the
same source with -DCTREF_F64: float64 throughout).

Part of the test infrastructure: used as the CPU baseline of bench.py
and by tests; never linked by the product.  ``-ffp-contract=off`` keeps
every operation rounded as written on both x86-64 and aarch64.
"""

from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "libctref.so"
OUT64 = HERE / "_build" / "libctref64.so"


def build(force: bool = False, f64: bool = False) -> Path:
    """Compile one variant (float32, or float64 with f64=True) if it is
    missing or older than the source; returns its path."""
    src = HERE / "ctref.c"
    out = OUT64 if f64 else OUT
    if out.exists() and not force and out.stat().st_mtime >= src.stat().st_mtime:
        return out
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the oracle")
    out.parent.mkdir(parents=True, exist_ok=True)
    cmd = [cc, "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC"]
    cmd += (["-DCTREF_F64"] if f64 else []) + ["-o", str(out), str(src), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    return out


def build_all(force: bool = False):
    return build(force), build(force, f64=True)


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
