"""Build libspirit_gb300.so in-tree: CUDA sources for sm_103a with nvcc, host C++ with g++.

    python -m spirit_gb300.build          (or spirit_gb300.build.build())

Translation units compile in parallel; objects go to spirit_gb300/_build/ and the library to
spirit_gb300/libspirit_gb300.so.  Rebuilds only what changed (timestamps incl. headers).
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libspirit_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _newest_header():
    hs = glob.glob(os.path.join(CSRC, "*.hpp")) + glob.glob(os.path.join(CSRC, "*.cuh"))
    return max((os.path.getmtime(h) for h in hs), default=0)


def _compile(src, cuda, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _newest_header()):
        return obj
    nvcc = os.path.join(cuda, "bin", "nvcc")
    if src.endswith(".cu"):
        cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC,-fopenmp,-O2", "-c", src, "-o", obj]
    else:
        cmd = ["g++", "-O2", "-fPIC", "-fopenmp", "-std=c++17", "-Wall", "-Wno-unused-function",
               "-I" + os.path.join(cuda, "include"), "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (src, r.stdout, r.stderr))
    if r.stderr.strip() and verbose:
        print(r.stderr)
    return obj


def build(verbose=False, jobs=None):
    cuda = _cuda_home()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, cuda, verbose), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        nvcc = os.path.join(cuda, "bin", "nvcc")
        cmd = [nvcc, ARCH, "-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lcudart", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
