"""Build the CUDA shared library of wendy_gb300 in-tree (sm_103a only).

    python -m wendy_gb300.build        # or wendy_gb300.build.build()

Each translation unit is compiled by nvcc in parallel, then linked into
wendy_gb300/_wendy_gb300.so next to this file.  No PyTorch, no cmake.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_wendy_gb300.so")
BUILD_DIR = os.path.join(HERE, "_build")
SOURCES = ["wg_kernels.cu", "wg_radix.cu", "wg_bucket.cu", "wg_api.cu", "wg_pool.cu",
           "wg_exact.cu", "wg_noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]
# the exact solver follows the reference's operation order without FMA contraction
FILE_FLAGS = {"wg_exact.cu": ["-fmad=false"]}


def nvcc():
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build wendy_gb300")


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "wendy_gb300.h"))
    cc = nvcc()
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([cc] + ARCH + FLAGS + FILE_FLAGS.get(src, []) + ["-c", s, "-o", o])
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, results):
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    if force or jobs or not _newer(OUT, objs):
        tmp = OUT + ".tmp"
        cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl",
                                                            "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
