"""Build the C/OpenMP restatement (oracle/ctref.c) into oracle/_build/libctref.so.

Part of the test infrastructure: used as the CPU baseline of bench.py
and by tests; never linked by the product.  ``-ffp-contract=off`` keeps
every float32 operation rounded as written on both x86-64 and aarch64.
"""

from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "libctref.so"


def build(force: bool = False) -> Path:
    src = HERE / "ctref.c"
    if OUT.exists() and not force and OUT.stat().st_mtime >= src.stat().st_mtime:
        return OUT
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the oracle")
    OUT.parent.mkdir(parents=True, exist_ok=True)
    cmd = [cc, "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC", "-o", str(OUT),
           str(src), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
