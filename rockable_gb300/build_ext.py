"""Build of the in-tree native libraries (librk_gpu.so).

The CUDA sources are compiled for sm_103a only.  The FP64 form is compiled
with --fmad=false: its results must be bit-identical to the reference CPU
arithmetic.  Objects are compiled in parallel; the shared library lands in
rockable_gb300/_lib/.
"""
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
BUILD = os.path.join(HERE, "_build", platform.machine())
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

# translation unit -> extra flags
UNITS = {
    "rk_prims.cu": [],
    "rk_step.cu": ["--fmad=false"],
    "rk_nl.cu": ["--fmad=false"],
    "rk_api.cu": ["--fmad=false"],
    "rk_mixed.cu": [],
    "rk_fast.cu": [],
    "rk_skin.cu": [],
    "rk_noalloc.cu": [],
}


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _compile(src, flags):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    srcp = os.path.join(CSRC, src)
    deps = [srcp] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "rk_gpu.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps if os.path.exists(d)):
        return obj
    # host code unfused too: the host-side arithmetic that feeds the FP64
    # form (body force parameters) must round like the reference's
    cmd = [nvcc(), GENCODE, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
           "-c", srcp, "-o", obj] + flags
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj


def build(verbose=False):
    """Compile every CUDA translation unit and link librk_gpu.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(*kv), UNITS.items()))
    out = os.path.join(LIBDIR, "librk_gpu.so")
    stamp = os.path.join(BUILD, "librk_gpu.so.stamp")
    if (not os.path.exists(out) or not os.path.exists(stamp)
            or any(os.path.getmtime(o) > os.path.getmtime(stamp) for o in objs)):
        cmd = [nvcc(), GENCODE, "-shared", "-o", out] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        open(stamp, "w").write(out + "\n")
    build_host(out)
    if verbose:
        print("built", out)
    return out


def build_host(gpu_lib):
    """librk_host.so (C++ host: conf I/O and plugin API over the C ABI) and the
    rockable-gb300 command-line runner."""
    hsrc = os.path.join(HERE, "host")
    cxx = shutil.which("g++") or "g++"
    host = os.path.join(LIBDIR, "librk_host.so")
    stamp = os.path.join(BUILD, "librk_host.so.stamp")
    srcs = [os.path.join(hsrc, "rk_host.cpp"), os.path.join(hsrc, "rk_extractors.cpp")]
    deps = srcs + [os.path.join(hsrc, "rk_host.hpp"), os.path.join(HERE, "..", "include", "rk_gpu.h"), gpu_lib]
    if not os.path.exists(stamp) or any(os.path.getmtime(d) > os.path.getmtime(stamp) for d in deps):
        cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-o", host] + srcs + \
              ["-L" + LIBDIR, "-lrk_gpu", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("host build failed:\n%s\n%s" % (r.stdout, r.stderr))
        cli = os.path.join(LIBDIR, "rockable-gb300")
        cmd = [cxx, "-O2", "-std=c++17", "-o", cli, os.path.join(hsrc, "rk_run.cpp"), "-L" + LIBDIR, "-lrk_host",
               "-lrk_gpu", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("runner build failed:\n%s\n%s" % (r.stdout, r.stderr))
        open(stamp, "w").write(host + "\n")
    build_packer()
    return host


def build_packer():
    """rk_pack, the CPU packer of the benchmark and test scenes: a standalone
    executable (no CUDA, no library of this package), so that a CPU-only
    process can build the same initial states as a GPU one."""
    src = os.path.join(HERE, "host", "rk_pack.cpp")
    exe = os.path.join(LIBDIR, "rk_pack")
    stamp = os.path.join(BUILD, "rk_pack.stamp")
    if os.path.exists(exe) and os.path.exists(stamp) and os.path.getmtime(stamp) >= os.path.getmtime(src):
        return exe
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-o", exe, src]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("packer build failed:\n%s\n%s" % (r.stdout, r.stderr))
    open(stamp, "w").write(exe + "\n")
    return exe


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
