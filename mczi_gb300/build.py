"""Builds the native parts of mczi_gb300 in-tree.

* ``mczi_gb300/lib/libmczi_gpu.so`` -- the CUDA kernels and the C ABI of
  ``include/mczi_gpu.h``, compiled for sm_103a only.
* ``mczi_gb300/lib/libmczi_gen.so`` -- the synthetic workload generator.

Translation units compile in parallel; the whole build takes well under a
minute.  Host code is portable C/C++ (x86_64 and aarch64 hosts).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB_DIR = PKG / "lib"
BUILD_DIR = PKG / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2,-fsigned-char",
              "-I", str(ROOT / "include")] + ARCH
CUDA_SOURCES = ["mc_pack.cu", "mc_scan.cu", "mc_partition.cu", "mc_count.cu", "mczi_api.cu", "zi.cu",
                "mc_pack_noalloc.cu", "mc_precount.cu", "simplitig.cu", "exchange.cu", "inflate.cu"]
CXX_SOURCES = ["host_io.cpp", "serve.cpp", "decompress.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build mczi_gb300")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _arch_guard() -> bool:
    """Objects from another host architecture (x86_64 vs aarch64) force a rebuild."""
    import platform
    BUILD_DIR.mkdir(exist_ok=True)
    stamp = BUILD_DIR / "host_arch"
    arch = platform.machine()
    if stamp.exists() and stamp.read_text() == arch:
        return False
    for o in BUILD_DIR.glob("*.o"):
        o.unlink()
    stamp.write_text(arch)
    return True


def build_gpu_lib(force: bool = False) -> Path:
    force = _arch_guard() or force
    LIB_DIR.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "mczi_gpu.h"]
    nv = nvcc()
    jobs = []
    objs = []
    for src in CUDA_SOURCES + CXX_SOURCES:
        s = CSRC / src
        if not s.exists():
            continue
        o = BUILD_DIR / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nv, *NVCC_FLAGS, "-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    lib = LIB_DIR / "libmczi_gpu.so"
    if force or jobs or _stale(lib, objs):
        _run([nv, "-shared", *ARCH, "-o", str(lib), *map(str, objs), "-lcudart", "-lpthread", "-ldl"])
    return lib


def build_gen_lib(force: bool = False) -> Path:
    LIB_DIR.mkdir(exist_ok=True)
    src = PKG / "gen" / "mczi_gen.c"
    lib = LIB_DIR / "libmczi_gen.so"
    if force or _stale(lib, [src]):
        cc = os.environ.get("CC", "gcc")
        _run([cc, "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fsigned-char", "-shared",
              "-o", str(lib), str(src), "-lm"])
    return lib


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        futs = [ex.submit(build_gpu_lib, force), ex.submit(build_gen_lib, force)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    import sys
    build_all(force="--force" in sys.argv)
    print("built", LIB_DIR)
