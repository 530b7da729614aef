"""In-tree build of libh2eri_gb300.so (host set-up + sm_103a kernels + C ABI).

Host sources are compiled with the system C/C++ compiler (portable flags only:
the same sources build on x86_64 and aarch64), CUDA sources with nvcc for
sm_103a, then linked with nvcc into h2p-eri_gb300/lib/libh2eri_gb300.so.
Objects go to h2p-eri_gb300/_build. Translation units compile in parallel.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))   # h2p-eri_gb300/
REPO = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
BUILD = os.path.join(PKG_ROOT, "_build")
LIBDIR = os.path.join(PKG_ROOT, "lib")
LIB = os.path.join(LIBDIR, "libh2eri_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INCS = ["-I" + os.path.join(REPO, "include"), "-I" + os.path.join(CSRC, "host"), "-I" + os.path.join(CSRC, "gpu")]
# -ffp-contract=off keeps host floating point identical between x86_64 and aarch64
HOST_FLAGS = ["-O3", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fvisibility=default"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    host = sorted(glob.glob(os.path.join(CSRC, "host", "*.c")) + glob.glob(os.path.join(CSRC, "host", "*.cpp")))
    cuda = sorted(glob.glob(os.path.join(CSRC, "gpu", "*.cu")))
    return host, cuda


def _headers():
    return (glob.glob(os.path.join(CSRC, "*", "*.h")) + glob.glob(os.path.join(CSRC, "*", "*.cuh"))
            + glob.glob(os.path.join(REPO, "include", "*.h")))


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc(), "-c", src, "-o", obj, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC,-fopenmp,-fvisibility=default"] + ARCH + INCS
    elif src.endswith(".cpp"):
        cmd = ["g++", "-c", src, "-o", obj, "-std=c++17"] + HOST_FLAGS + INCS
    else:
        cmd = ["gcc", "-c", src, "-o", obj, "-std=gnu11"] + HOST_FLAGS + INCS
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return obj


def build(verbose=False, jobs=None):
    """Compile every translation unit and link the shared library. Returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    host, cuda = _sources()
    srcs = cuda + host
    jobs = jobs or min(len(srcs), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [_nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fopenmp", "-lgomp", "-lpthread"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
