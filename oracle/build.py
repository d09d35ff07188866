"""Build recipe of the oracle (test infrastructure): the C restatement in oracle.c -> _build/liboracle.so.

Only tests/, __graft_entry__.smoke() and the CPU-baseline legs of bench.py load this library.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle.so"


def build(force: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    src = HERE / "oracle.c"
    deps = [src, HERE / "oracle.h", HERE.parent / "include" / "gpe.h"]
    if force or not OUT.exists() or any(d.stat().st_mtime > OUT.stat().st_mtime for d in deps):
        cc = shutil.which("gcc") or "cc"
        cmd = [cc, "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(OUT), str(src), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
