"""In-tree build of libsisgpu.so for sm_103a (nvcc, no cmake).

Each translation unit is compiled in parallel, then linked with the static
CUDA runtime so that the library needs nothing beyond the NVIDIA kernel-mode
and user-mode driver libraries (libcuda).
Objects go to ``_build/``, the library to ``sis_gb300/_lib/``.
"""
from __future__ import annotations

import hashlib
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = ROOT / "_build"
LIB = PKG / "_lib" / "libsisgpu.so"
SOURCES = ["kernels.cu", "lists.cu", "remd.cu", "api.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-Wno-deprecated-declarations,-ffp-contract=off", "-diag-suppress", "1444"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


STAMP = LIB.with_suffix(".so.sha256")


def source_key(cc: str) -> str:
    """Hash of every source, the flags, the compiler path and the machine:
    the library is rebuilt whenever any of them differs from the build that
    made it (file times are not trusted: copies between machines keep them)."""
    h = hashlib.sha256()
    for p in sorted(CSRC.glob("*")) + [ROOT / "include" / "sis_gpu.h"]:
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join([cc, *FLAGS, *ARCH, platform.machine()]).encode())
    return h.hexdigest()


def build_lib(verbose: bool = False, force: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    LIB.parent.mkdir(exist_ok=True)
    cc = nvcc()
    key = source_key(cc)
    if LIB.exists() and not force and STAMP.exists() and STAMP.read_text().strip() == key:
        return LIB

    def compile_one(src: str):
        out = OBJ / (Path(src).stem + ".o")
        cmd = [cc, *FLAGS, *ARCH, "-c", str(CSRC / src), "-o", str(out)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return out

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-shared", *ARCH, "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    STAMP.write_text(key + "\n")
    return LIB


if __name__ == "__main__":
    print(build_lib(verbose=True, force="--force" in sys.argv))
