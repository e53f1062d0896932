"""Builds the native parts in-tree:

* golaypair_gb300/_build/libgolaypair_gb300.so -- the CUDA kernels (sm_103a)
  and the C ABI declared in include/golaypair_gb300.h;
* golaypair_gb300/_build/golay -- the command line driver that mirrors the
  reference's `main` (src/main.cpp), linked against the library.

Translation units compile in parallel; one -gencode (sm_103a) only.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libgolaypair_gb300.so")
CLI = os.path.join(OUT, "golay")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
           "--expt-relaxed-constexpr", "-I" + os.path.join(REPO, "include")]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, ptxas_info=False):
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        [os.path.join(REPO, "include", "golaypair_gb300.h")]
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    jobs = []
    objs = []
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if ptxas_info or _stale(o, [s] + headers):
            cmd = [cc] + ARCH + NVFLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + ["-c", s, "-o", o]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose or ptxas_info:
                sys.stdout.write(out)
    if jobs or not os.path.exists(LIB):
        _run([cc] + ARCH + ["-shared", "-o", LIB] + objs + ["-cudart", "static", "-lpthread", "-ldl", "-lrt"])
    host_srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    if host_srcs and _stale(CLI, host_srcs + [LIB] + glob.glob(os.path.join(HOST, "*.h"))):
        _run(["g++", "-O2", "-std=c++20", "-Wall", "-I" + os.path.join(REPO, "include"), "-o", CLI] + host_srcs +
             ["-L" + OUT, "-lgolaypair_gb300", "-Wl,-rpath,$ORIGIN", "-lpthread"])
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
