"""Compile the sm_103a kernels and the C ABI into gisapr_gb300/_native/.

    python -m gisapr_gb300.build_native [--force] [--verbose]

Each .cu translation unit is compiled in parallel with one -gencode
(arch=compute_103a, code=sm_103a) and linked into libgisapr_gb300.so with
cuFFT and the shared CUDA runtime. Object files and the library stay in the
source tree (git-ignored), so the library is found next to the package.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "csrc"
OUT = PKG / "_native"
LIB = OUT / "libgisapr_gb300.so"
INCLUDE = PKG.parent / "include"
SOURCES = ["splat.cu", "project.cu", "volfft.cu", "particles.cu", "correlate.cu", "correlate_tc.cu", "restraint.cu",
           "ingest.cu", "abi.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> Path:
    for key in ("CUDA_HOME", "CUDA_PATH"):
        if os.environ.get(key):
            return Path(os.environ[key])
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _digest() -> str:
    h = hashlib.sha256()
    for p in sorted(list(SRC.glob("*.cu")) + list(SRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join(ARCH).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    stamp = OUT / "build.stamp"
    digest = _digest()
    if LIB.exists() and stamp.exists() and stamp.read_text() == digest and not force:
        return LIB
    home = cuda_home()
    nvcc = str(home / "bin" / "nvcc")
    common = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-I", str(INCLUDE), "-I", str(SRC)]
    if verbose:
        common += ["-Xptxas", "-v"]

    def compile_one(name: str):
        obj = OUT / (Path(name).stem + ".o")
        cmd = common + ["-c", str(SRC / name), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    libdir = home / "lib64"
    if not libdir.exists():
        libdir = home / "lib"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "shared",
           "-L", str(libdir), "-lcufft", "-Xlinker", f"-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(digest)
    return LIB


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))


if __name__ == "__main__":
    main()
