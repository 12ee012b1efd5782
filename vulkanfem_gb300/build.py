"""Build libvfem.so (the C-ABI CUDA library) in-tree for sm_103a.

Translation units are compiled in parallel with nvcc and linked into
``vulkanfem_gb300/_build/libvfem.so``.  Nothing is installed outside the tree.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libvfem.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["setup.cpp", "setup_gpu.cu", "kernels.cu", "matvec_tc.cu", "transfer_tma.cu", "api.cu", "unet.cu"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvfem")


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def build(force=False, verbose=False, extra_flags=()):
    """Compile and link; returns the library path.  Raises on failure."""
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    headers = _headers()
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", CSRC, "-I", INCLUDE] + list(extra_flags)
    jobs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            cmd = [nv] + ARCH + common + ["-c", path, "-o", obj]
            if src.endswith(".cpp"):
                cmd = [nv] + common + ["-x", "c++", "-c", path, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return r.stderr

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for msg in ex.map(run, jobs):
            if verbose and msg:
                print(msg)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcusolver", "-lcublas", "-lcudart"]
        run(cmd)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
