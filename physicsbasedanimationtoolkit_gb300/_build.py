"""In-tree build of the CUDA library ``_lib/libpbat_gb300.so`` (sm_103a only).

Translation units are compiled in parallel with nvcc / g++ and linked with nvcc; the outputs stay
inside the package directory (git-ignored).  A rebuild happens only when a source is newer than
the library.
"""

from __future__ import annotations

import os
import pathlib
import shutil
import subprocess
import sys

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUT_DIR = PKG / "_lib"
OBJ_DIR = OUT_DIR / "obj"
LIB = OUT_DIR / "libpbat_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-lineinfo",
    "-O3",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-fvisibility=hidden",
    f"-I{INCLUDE}",
    f"-I{CSRC}",
]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fvisibility=hidden", f"-I{INCLUDE}", f"-I{CSRC}"]

CUDA_SOURCES = ["vbd_kernels.cu", "batched.cu", "vbd_capi.cu", "adjoint.cu", "anderson.cu", "nesterov.cu", "trust_region.cu", "lbvh.cu", "lbvh_capi.cu", "contact.cu", "contact_capi.cu"]
CXX_SOURCES = ["vbd_construct.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def _sources():
    return [CSRC / s for s in CUDA_SOURCES + CXX_SOURCES] + sorted(CSRC.glob("*.cuh")) + sorted(
        CSRC.glob("*.h")
    ) + sorted(INCLUDE.glob("*.h"))


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _sources())


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    """Compile and link the library; returns its path."""
    if not force and up_to_date():
        return LIB
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    cxx = os.environ.get("CXX", "g++")
    jobs = []
    objs = []
    for s in CUDA_SOURCES:
        o = OBJ_DIR / (s + ".o")
        objs.append(o)
        jobs.append([nvcc, *NVCC_FLAGS, "-c", str(CSRC / s), "-o", str(o)])
    for s in CXX_SOURCES:
        o = OBJ_DIR / (s + ".o")
        objs.append(o)
        jobs.append([cxx, *CXX_FLAGS, "-c", str(CSRC / s), "-o", str(o)])
    procs = [
        subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True) for j in jobs
    ]
    failed = []
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        if verbose and out:
            sys.stdout.write(out)
        if p.returncode != 0:
            failed.append((j, out))
    if failed:
        msg = "\n".join(" ".join(j) + "\n" + out for j, out in failed)
        raise RuntimeError(f"library build failed:\n{msg}")
    tmp = LIB.with_suffix(".so.tmp")
    link = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + " ".join(link) + "\n" + r.stdout)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
