"""In-tree build of libnqes.so (CUDA, sm_103a) and the drop-in executables.

    python nqes-trapped-ion_gb300/build.py [--verbose]

Translation units are compiled in parallel with one -gencode for sm_103a and
linked into nqes-trapped-ion_gb300/lib/libnqes.so. No cmake, no torch
extension machinery: the library is a plain C-ABI shared object.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")

SOURCES = ["kernels_sample.cu", "kernels_solve.cu", "nqes_api.cu", "sv_static.cu"]
HEADERS = ["nqes_math.cuh", "pcg64.cuh", "nqes_internal.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnqes")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    obj = os.path.join(OBJDIR, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "nqes.h")]
    if not _stale(obj, deps):
        return obj
    cmd = [nvcc(), "-std=c++17", *ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE,
           "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build_library(verbose=False):
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    lib = os.path.join(LIBDIR, "libnqes.so")
    if _stale(lib, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", lib, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of libnqes.so failed:\n{r.stderr}")
    return lib


def main():
    lib = build_library(verbose="--verbose" in sys.argv)
    print(lib)


if __name__ == "__main__":
    main()
