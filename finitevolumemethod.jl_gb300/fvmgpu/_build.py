"""Builds libfvmgpu.so (sm_103a) in-tree, in parallel, without cmake.

Host sources compile with g++ (-ffp-contract=off so the geometry rounds the same on x86
and Arm), device sources with nvcc for sm_103a only; cudart is linked statically so the
library loads with ctypes alone.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG.parent / "csrc"
INCLUDE = PKG.parent.parent / "include"
LIBDIR = PKG / "_lib"
LIBNAME = "libfvmgpu.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


# the device mesh build rounds like the host one (-ffp-contract=off there): no FMA contraction
NVCC_FILE_FLAGS = {"fvm_mesh_dev.cu": ["-fmad=false"], "fvm_post.cu": ["-fmad=false"]}


def sources():
    return sorted(CSRC.glob("*.cpp")), sorted(CSRC.glob("*.cu"))


def lib_path() -> Path:
    return LIBDIR / LIBNAME


def _stale(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every source and link libfvmgpu.so; returns its path."""
    target = lib_path()
    if not force and not _stale(target):
        return target
    cuda = cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    objdir = LIBDIR / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    cpp, cu = sources()
    inc = [f"-I{INCLUDE}", f"-I{cuda / 'include'}"]
    jobs = []
    for src in cpp:
        obj = objdir / (src.stem + ".o")
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                     *inc, "-c", str(src), "-o", str(obj)])
    for src in cu:
        obj = objdir / (src.stem + ".cu.o")
        jobs.append([nvcc, "-std=c++17", "-O3", ARCH, "-lineinfo", "-Xcompiler", "-fPIC", *inc,
                     *NVCC_FILE_FLAGS.get(src.name, []), "-c", str(src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return cmd[-1]

    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        objs = list(ex.map(run, jobs))
    libdirs = [cuda / "lib64", cuda / "targets" / "sbsa-linux" / "lib", cuda / "targets" / "x86_64-linux" / "lib"]
    link = ["g++", "-shared", "-o", str(target) + ".tmp", *objs]
    link += [f"-L{d}" for d in libdirs if d.exists()]
    link += ["-lcudart_static", "-ldl", "-lrt", "-lpthread"]
    run(link)
    os.replace(str(target) + ".tmp", target)
    return target


if __name__ == "__main__":
    print(build(force=True, verbose=True))
