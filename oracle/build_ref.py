"""Builds the reference's own kernels headless for sm_103a — test infrastructure for the parity tests and the
reference-CUDA timing leg, never part of the engine.

libs/cuda-engine/source/PBF.cu and MPM.cu and libs/render/source/cuda-render.cu (its backgroundKernel and
drawKernel, which include no graphics headers) are compiled unmodified from the reference checkout into
device-only cubins under oracle/_ref/ (git-ignored; the cubins travel to the GPU machine, where the reference
sources do not exist). The engine's headless common/ headers (gpu-physics-engine_gb300/compat/common) replace
the reference's MSVC-only macros.h and its umbrella.h and supply its constants.h values, with the scene size
and capacities overridable by -D.

The checkout is read from the directory in the environment variable GPE_REFERENCE_DIR, by default the
reference's location in the build container. Where the sources are absent (the GPU machine), prebuilt cubins are
used as they are.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
REF = Path(os.environ.get("GPE_REFERENCE_DIR", "/root/reference"))
ENGINE_SRC = REF / "libs" / "cuda-engine" / "source"
ENGINE_INC = REF / "libs" / "cuda-engine" / "include"
RENDER_SRC = REF / "libs" / "render" / "source"
RENDER_INC = REF / "libs" / "render" / "include"

# (file stem, kernel source, -D overrides)
VARIANTS = [
    ("PBF_ref_12x6_m320", ENGINE_SRC / "PBF.cu", {}),
    ("PBF_ref_32x32_m320", ENGINE_SRC / "PBF.cu", {"GPE_REF_SCENE_X": 32, "GPE_REF_SCENE_Y": 32}),
    ("MPM_ref_12x6_n400000", ENGINE_SRC / "MPM.cu", {}),
    ("MPM_ref_64x64_n4194304", ENGINE_SRC / "MPM.cu", {"GPE_REF_SCENE_X": 64, "GPE_REF_SCENE_Y": 64,
                                                       "GPE_REF_MPM_ATOMS": 4194304}),
    ("render_ref_12x6", RENDER_SRC / "cuda-render.cu", {}),
]


def _nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def build(force: bool = False) -> list[Path]:
    OUT.mkdir(exist_ok=True)
    outs = [OUT / f"{stem}.cubin" for stem, _, _ in VARIANTS]
    if not ENGINE_SRC.exists():
        return [o for o in outs if o.exists()]
    # an include root holding only common/ (the package's compat/ also holds a cuda-engine/cuda-engine.h
    # that must not shadow the reference's own)
    shim = sorted((HERE.parent / "gpu-physics-engine_gb300" / "compat" / "common").glob("*.h"))
    common = OUT / "inc"
    (common / "common").mkdir(parents=True, exist_ok=True)
    for h in shim:
        dst = common / "common" / h.name
        if not dst.exists() or dst.read_bytes() != h.read_bytes():
            shutil.copyfile(h, dst)
    jobs = []
    for (stem, src, defs), out in zip(VARIANTS, outs):
        if not src.exists():
            continue
        deps = [src, *shim]
        if not force and out.exists() and all(d.stat().st_mtime <= out.stat().st_mtime for d in deps):
            continue
        cmd = [_nvcc(), "-cubin", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo",
               "-diag-suppress", "177,1675", "-I", str(common), "-I", str(ENGINE_INC), "-I", str(RENDER_INC),
               *[f"-D{k}={v}" for k, v in defs.items()], "-o", str(out), str(src)]
        jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference kernel build failed: " + " ".join(cmd) + "\n" + r.stderr)

    with ThreadPoolExecutor(max_workers=4) as ex:
        list(ex.map(run, jobs))
    return outs


if __name__ == "__main__":
    for p in build(force=True):
        print(p)
