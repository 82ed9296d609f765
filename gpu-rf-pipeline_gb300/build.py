"""Build recipe for librfx.so (the CUDA kernels + C ABI) and the rfgpu command-line tool.

    python gpu-rf-pipeline_gb300/build.py          # or __graft_entry__.build()

Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, into gpu-rf-pipeline_gb300/_build/;
the shared library lands in gpu-rf-pipeline_gb300/lib/ and the CLI in gpu-rf-pipeline_gb300/bin/.
Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
BUILD = PKG / "_build"
LIB = PKG / "lib" / "librfx.so"
# The C++ drop-in layer (host/*.cpp without the CLI's main): the project's device_ops.hpp /
# ops.hpp / stream.hpp functions over the C ABI, for programs written against those headers.
HOSTLIB = PKG / "lib" / "librfxhost.a"
CLI = PKG / "bin" / "rfgpu"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def nvcc() -> str:
    found = shutil.which("nvcc")
    return found if found else str(cuda_home() / "bin" / "nvcc")


def _newest_header(folder: Path) -> float:
    stamps = [p.stat().st_mtime for p in folder.glob("*.cuh")]
    stamps += [p.stat().st_mtime for p in folder.glob("*.hpp")]
    stamps += [p.stat().st_mtime for p in INCLUDE.glob("*.h")]
    return max(stamps) if stamps else 0.0


def _compile(src: Path, obj: Path, flags: list[str]) -> tuple[Path, str]:
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I", str(INCLUDE), "-I", str(CSRC), *flags, "-c", str(src), "-o", str(obj)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{' '.join(cmd)}\n{proc.stderr}")
    return obj, proc.stderr


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    CLI.parent.mkdir(parents=True, exist_ok=True)
    header_time = max(_newest_header(CSRC), _newest_header(HOST) if HOST.exists() else 0.0)
    jobs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".o")
        if not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, header_time):
            jobs.append((src, obj, []))
    host_srcs = sorted(HOST.glob("*.cpp")) if HOST.exists() else []
    for src in host_srcs:
        obj = BUILD / ("host_" + src.stem + ".o")
        if not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, header_time):
            jobs.append((src, obj, ["-I", str(HOST), "-x", "cu"]))
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as pool:
        for obj, log in pool.map(lambda j: _compile(*j), jobs):
            if verbose and log.strip():
                print(log, file=sys.stderr)
    lib_objs = [BUILD / (s.stem + ".o") for s in sorted(CSRC.glob("*.cu"))]
    cuda_lib = cuda_home() / "lib64"
    if not LIB.exists() or LIB.stat().st_mtime < max(o.stat().st_mtime for o in lib_objs):
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", str(LIB),
               *map(str, lib_objs), "-lcufft", "-Xlinker", f"-rpath,{cuda_lib}"]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{proc.stderr}")
    host_objs = [BUILD / ("host_" + s.stem + ".o") for s in host_srcs]
    layer_objs = [o for o in host_objs if o.name != "host_main.o"]
    if layer_objs and (not HOSTLIB.exists()
                       or HOSTLIB.stat().st_mtime < max(o.stat().st_mtime for o in layer_objs)):
        HOSTLIB.unlink(missing_ok=True)
        proc = subprocess.run(["ar", "rcs", str(HOSTLIB), *map(str, layer_objs)],
                              capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"ar failed:\n{proc.stderr}")
    if host_objs and (not CLI.exists()
                      or CLI.stat().st_mtime < max(o.stat().st_mtime
                                                   for o in host_objs + [LIB])):
        cmd = [nvcc(), *ARCH, "-cudart", "shared", "-o", str(CLI), *map(str, host_objs),
               "-L", str(LIB.parent), "-lrfx", "-lcufft",
               "-Xlinker", f"-rpath,{LIB.parent}", "-Xlinker", f"-rpath,{cuda_lib}"]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{proc.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
