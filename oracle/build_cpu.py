"""Build the oracle's C/OpenMP restatements (``oracle/cpu_ref.c``,
``oracle/cpu_burgers.c``) into
``oracle/_build/libexc_cpu_ref.so`` with gcc.  Test infrastructure only."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "cpu_ref.c"
SRCS = [SRC, HERE / "cpu_burgers.c"]
OUT = HERE / "_build" / "libexc_cpu_ref.so"


def build() -> Path | None:
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        return None
    OUT.parent.mkdir(exist_ok=True)
    if OUT.exists() and OUT.stat().st_mtime > max(s.stat().st_mtime for s in SRCS):
        return OUT
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [cc, "-O3", "-fopenmp", "-shared", "-fPIC", "-std=gnu11", *map(str, SRCS), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    tmp.replace(OUT)
    return OUT


if __name__ == "__main__":
    print(build())
