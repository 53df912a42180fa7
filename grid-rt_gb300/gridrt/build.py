"""Compiles libgridrt.so (the CUDA kernels + C ABI) in-tree for sm_103a.

Each .cu file is compiled in parallel to an object, then linked into
grid-rt_gb300/gridrt/_lib/libgridrt.so.  The build is incremental: an object
is rebuilt when its source or a header in csrc/ or include/ is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                      # grid-rt_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libgridrt.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _newest(paths) -> float:
    return max((os.path.getmtime(p) for p in paths if os.path.exists(p)), default=0.0)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    hdr_time = _newest(headers)
    objs = []
    jobs = []
    for src in sources:
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time):
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-I", INCLUDE, "-c", src, "-o", obj]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            futs = [ex.submit(subprocess.run, cmd, capture_output=True, text=True) for cmd in jobs]
            for cmd, f in zip(jobs, futs):
                r = f.result()
                if verbose or r.returncode:
                    print(" ".join(cmd))
                    print(r.stdout, r.stderr)
                if r.returncode:
                    raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    if jobs or not os.path.exists(LIB):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            print(" ".join(cmd), r.stdout, r.stderr)
            raise RuntimeError("link failed")
    build_tools()
    return LIB


TOOLS = {
    # C++ driver of the plugin mirror (include/gridrt_rtp.hpp), used by tests
    "rtp_adapter_check": os.path.join(REPO, "tests", "cpp", "rtp_adapter_check.cpp"),
}


def tool_path(name: str) -> str:
    return os.path.join(OUT_DIR, name)


def build_tools() -> None:
    for name, src in TOOLS.items():
        out = tool_path(name)
        if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(src), os.path.getmtime(LIB),
                                                                   _newest(glob.glob(os.path.join(INCLUDE, "*")))):
            continue
        cuda_lib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "lib64") \
            if os.path.isabs(nvcc()) else "/usr/local/cuda/lib64"
        cmd = ["g++", "-O2", "-std=c++17", "-I", INCLUDE, src, "-o", out, "-L", OUT_DIR, "-lgridrt",
               f"-Wl,-rpath,{OUT_DIR}", "-L", cuda_lib, "-lcudart", f"-Wl,-rpath,{cuda_lib}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            print(" ".join(cmd), r.stdout, r.stderr)
            raise RuntimeError(f"building {name} failed")


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
