"""In-tree build of libfullmag_fdm.so for sm_103a (nvcc, no cmake).

Each translation unit compiles in its own nvcc process (in parallel), then one
link step produces fullmag_gb300/_build/libfullmag_fdm.so.  The library links only
the CUDA runtime; no torch types cross its C ABI.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libfullmag_fdm.so"
SOURCES = ["row_pass.cu", "columns.cu", "engine.cu", "newell.cu", "adjoint.cu", "noalloc.cu", "extra_field.cu", "fp64.cu"]
# the cuFFT + unfused measurement baseline: a separate library, never linked into the product
PLAIN_SOURCES = ["plain_baseline.cu"]
PLAIN_LIB = OUT / "libfullmag_fdm_plain.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfullmag_fdm.so")
    return p


def _stale() -> bool:
    if not LIB.exists() or not PLAIN_LIB.exists():
        return True
    t = min(LIB.stat().st_mtime, PLAIN_LIB.stat().st_mtime)
    deps = [SRC / s for s in SOURCES + PLAIN_SOURCES if (SRC / s).exists()]
    deps += list(SRC.glob("*.cuh")) + list(SRC.glob("*.h")) + [PKG.parent / "include" / "fullmag_fdm.h"]
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale():
        return LIB
    OUT.mkdir(parents=True, exist_ok=True)
    cc = nvcc()
    srcs = [s for s in SOURCES + PLAIN_SOURCES if (SRC / s).exists()]

    def compile_one(s: str) -> Path:
        obj = OUT / (Path(s).stem + ".o")
        cmd = [cc, *FLAGS, *ARCH, "-c", str(SRC / s), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {s}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = dict(zip(srcs, ex.map(compile_one, srcs)))

    def link(out: Path, parts, libs):
        tmp = out.with_name(out.name + ".tmp")
        cmd = [cc, "-shared", *ARCH, *map(str, parts), "-o", str(tmp), *libs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of {out.name} failed:\n{r.stderr}")
        os.replace(tmp, out)

    link(LIB, [objs[s] for s in SOURCES if s in objs], ["-lcudart"])
    # the plain baseline builds its tensor with newell.cu, whose periodic builder uses the
    # FP64 line transforms of fp64.cu
    link(PLAIN_LIB, [objs[s] for s in PLAIN_SOURCES if s in objs] + [objs["newell.cu"], objs["fp64.cu"]],
         ["-lcufft", "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
