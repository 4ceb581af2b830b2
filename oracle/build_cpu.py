"""Build the oracle's C/OpenMP restatement (``oracle/cpu_ref.c``) into
``oracle/_build/libexc_cpu_ref.so`` with gcc.  Test infrastructure only."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "cpu_ref.c"
OUT = HERE / "_build" / "libexc_cpu_ref.so"


def build() -> Path | None:
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        return None
    OUT.parent.mkdir(exist_ok=True)
    if OUT.exists() and OUT.stat().st_mtime > SRC.stat().st_mtime:
        return OUT
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [cc, "-O3", "-fopenmp", "-shared", "-fPIC", "-std=gnu11", str(SRC), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    tmp.replace(OUT)
    return OUT


if __name__ == "__main__":
    print(build())
