"""In-tree build of the CUDA library (libmocgpu.so) for sm_103a.

Host C++ sources are compiled with g++, CUDA sources with nvcc
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked into
``mocc_gb300/_build/libmocgpu.so``. A content hash of the sources and flags
skips the rebuild when nothing changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "csrc"
OUT = PKG / "_build"
INCLUDE = PKG.parent / "include"
LIB_NAME = "libmocgpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and Path(cand, "bin", "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _sources():
    host = sorted((SRC / "host").glob("*.cpp"))
    dev = sorted((SRC / "device").glob("*.cu")) + [SRC / "capi.cu"]
    headers = sorted(SRC.rglob("*.hpp")) + sorted(SRC.rglob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    return host, dev, headers


def _flags(ch: Path):
    cxx = ["g++", "-std=c++17", "-O2", "-fPIC", "-Wall", f"-I{ch / 'include'}", f"-I{INCLUDE}"]
    nv = [str(ch / "bin" / "nvcc"), "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", *ARCH,
          f"-I{INCLUDE}", "--expt-relaxed-constexpr"]
    # extra nvcc flags, e.g. -DMOCGPU_SWEEP_ROWS=4 to build another sweep chunk shape
    nv += os.environ.get("MOCGPU_NVCC_EXTRA", "").split()
    return cxx, nv


def _digest(files, flags) -> str:
    h = hashlib.sha256()
    for f in files:
        h.update(str(f.relative_to(PKG.parent)).encode())
        h.update(f.read_bytes())
    h.update(" ".join(" ".join(x) for x in flags).encode())
    return h.hexdigest()


def build_library(force: bool = False, verbose: bool = False) -> Path:
    """Compiles libmocgpu.so if needed and returns its path."""
    ch = cuda_home()
    host, dev, headers = _sources()
    cxx, nv = _flags(ch)
    digest = _digest(host + dev + headers, (cxx, nv))
    OUT.mkdir(exist_ok=True)
    lib = OUT / LIB_NAME
    stamp = OUT / "libmocgpu.stamp"
    if not force and lib.exists() and stamp.exists() and stamp.read_text() == digest:
        return lib
    objs, jobs = [], []
    for s in host:
        o = OUT / (s.stem + ".o")
        objs.append(o)
        jobs.append(cxx + ["-c", str(s), "-o", str(o)])
    for s in dev:
        o = OUT / (s.stem + ".cu.o")
        objs.append(o)
        jobs.append(nv + ["-c", str(s), "-o", str(o)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        list(ex.map(run, jobs))
    tmp = OUT / (LIB_NAME + ".tmp")
    run([str(ch / "bin" / "nvcc"), "-shared", *ARCH, "-o", str(tmp)] + [str(o) for o in objs])
    tmp.replace(lib)
    stamp.write_text(digest)
    return lib


if __name__ == "__main__":
    print(build_library(force=True, verbose=True))
