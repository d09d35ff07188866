"""Build recipe for libgpe.so (the CUDA engine behind include/gpe.h), compiled in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into one shared library next to this
file. The library is the product: the Python package `gpe` loads it and fails loudly when it is missing.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libgpe.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["capi.cu", "sort.cu", "pbf.cu", "mpm.cu", "mlp.cu", "render.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "gpe.h"]
    cc = nvcc()
    flags = ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
             "-I", str(PKG.parent / "include")]
    jobs = []
    objs = []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            jobs.append([cc, *flags, "-c", str(s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([cc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"])
    build_compat(cc, flags, force)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


COMPAT = PKG / "compat"
COMPAT_LIB = PKG / "libgpe_compat.so"
EXAMPLES = ["pbf_headless", "mpm_headless"]


def build_compat(cc: str, flags: list[str], force: bool = False) -> None:
    """libgpe_compat.so (the reference's cuda-engine.h on top of libgpe.so) and the headless example drivers."""
    headers = [COMPAT / "cuda-engine" / "cuda-engine.h", *sorted((COMPAT / "common").glob("*.h")),
               PKG.parent / "include" / "gpe.h"]
    inc = ["-I", str(COMPAT)]
    rpath = ["-Xlinker", "-rpath", "-Xlinker", str(PKG)]
    src = COMPAT / "cuda-engine.cu"
    obj = BUILD / "compat_cuda_engine.o"
    if force or _stale(obj, [src, *headers]):
        _run([cc, *flags, *inc, "-c", str(src), "-o", str(obj)])
    if force or _stale(COMPAT_LIB, [obj, LIB]):
        _run([cc, *ARCH, "-shared", "-o", str(COMPAT_LIB), str(obj), "-L", str(PKG), "-lgpe", "-lcudart", *rpath])
    (COMPAT / "bin").mkdir(exist_ok=True)
    jobs = []
    for ex in EXAMPLES:
        s = COMPAT / "examples" / f"{ex}.cpp"
        out = COMPAT / "bin" / ex
        if force or _stale(out, [s, COMPAT_LIB, *headers]):
            jobs.append([cc, "-std=c++17", "-O2", *inc, "-I", str(PKG.parent / "include"), str(s), "-o", str(out),
                         "-L", str(PKG), "-lgpe_compat", "-lgpe", "-lcudart", *rpath])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
