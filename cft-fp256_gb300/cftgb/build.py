"""Build the library in-tree: nvcc compiles every translation unit under
csrc/ for sm_103a in parallel, then links lib/libcft_gb300.so.

Kept free of cmake and of torch's extension machinery: the product is a
plain C-ABI shared library, and the same two nvcc command shapes build it
on an x86 build host (cross-compiling the device code) and on the Arm GPU
host.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent.parent          # cft-fp256_gb300/
ROOT = PKG.parent                                     # repository root
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "lib" / "libcft_gb300.so"
TOOL = PKG / "lib" / "cftg-asm"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "-lineinfo", "-I", str(ROOT / "include")]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcft_gb300")


def sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _compile(src):
    out = OBJ / (src.name + ".o")
    deps = [src] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))
    if out.exists() and out.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return out, ""
    cmd = [nvcc()] + ARCH + COMMON + ["-c", str(src), "-o", str(out)]
    if src.suffix == ".cu":
        cmd += ["-Xptxas", "-warn-spills"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{p.stdout}\n{p.stderr}")
    return out, p.stderr


def build_lib(verbose=False):
    OBJ.mkdir(parents=True, exist_ok=True)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        results = list(ex.map(_compile, srcs))
    objs = [r[0] for r in results]
    if verbose:
        for _, log in results:
            if log.strip():
                print(log, file=sys.stderr)
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + ["-lcuda"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed:\n{p.stdout}\n{p.stderr}")
    build_tool()
    return LIB


def build_tool():
    """cftg-asm, the assembler command, over the library (host code only)."""
    src = CSRC / "tools" / "cftg_asm.cpp"
    if TOOL.exists() and TOOL.stat().st_mtime >= max(src.stat().st_mtime, LIB.stat().st_mtime):
        return TOOL
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(src), "-o", str(TOOL),
           "-L", str(LIB.parent), "-lcft_gb300", "-Wl,-rpath,$ORIGIN"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"cftg-asm build failed:\n{p.stdout}\n{p.stderr}")
    return TOOL


def build_oracle():
    """The checker's C restatement (oracle/). Built here too so that tests
    and the CPU baseline find it; the shipped library never links it."""
    p = subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "port"], capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{p.stdout}\n{p.stderr}")
    return ROOT / "oracle" / "_build" / "libsfport.so"


if __name__ == "__main__":
    print(build_lib(verbose=True))
    print(build_oracle())
