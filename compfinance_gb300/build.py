"""Build libcfgpu.so in-tree: every CUDA translation unit for sm_103a with nvcc, the host
C++ with g++ (-ffp-contract=off so host doubles round like the reference's), compiled in
parallel and linked with nvcc into compfinance_gb300/libcfgpu.so.

    python3 -m compfinance_gb300.build [--force]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcfgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def sources():
    cu = sorted(f for f in os.listdir(SRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(SRC) if f.endswith(".cpp"))
    return cu, cpp


def _stale(obj, src_files):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(f) > t for f in src_files)


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    inc = os.path.join(_cuda_home(), "include")
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(HERE, "data", "sobol_joe_kuo.inc"),
                os.path.join(os.path.dirname(HERE), "include", "cfgpu.h")]
    cu, cpp = sources()
    jobs = []
    objs = []
    for f in cu:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
                         "-diag-suppress", "128", "-c", src, "-o", obj])
    for f in cpp:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                         "-I", inc, "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        bad = [(c, r) for c, r in zip(jobs, results) if r.returncode != 0]
        for c, r in zip(jobs, results):
            if verbose or r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
        if bad:
            raise RuntimeError("build failed: " + " ".join(bad[0][0]))
    if force or jobs or not os.path.exists(LIB):
        cmd = [nvcc, "-shared", *ARCH, "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
