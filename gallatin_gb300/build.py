"""In-tree build of libgallatin_gb300.so for sm_103a (nvcc, no cmake).

    python -m gallatin_gb300.build        # or gallatin_gb300.build.build()

Translation units compile in parallel, then link into one shared library next
to this file.  Outputs are git-ignored.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgallatin_gb300.so")
SOURCES = ["gal_lib.cu", "gal_bench.cu", "gal_noalloc.cu", "gal_serve.cu", "gal_tables.cu", "gal_server.cu"]
HEADERS = [
    os.path.join(ROOT, "include", "gallatin_gb300.h"),
    os.path.join(ROOT, "include", "gallatin_gb300", "gal_device.cuh"),
    os.path.join(CSRC, "gal_batch.cuh"),
    os.path.join(CSRC, "churn.cuh"),
    os.path.join(CSRC, "workload.cuh"),
    os.path.join(CSRC, "gal_internal.h"),
    os.path.join(CSRC, "gal_server.cuh"),
]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include")]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + HEADERS):
            jobs.append([nvcc()] + NVCC_FLAGS + ARCH + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")

    dropin_src = os.path.join(ROOT, "tests", "dropin", "dropin_test.cu")
    dropin_lib = os.path.join(ROOT, "tests", "dropin", "libdropin_test.so")
    dropin_headers = HEADERS + [os.path.join(ROOT, "include", "gallatin", "allocators", h)
                                for h in ("gallatin.cuh", "global_allocator.cuh")]
    with ThreadPoolExecutor(max_workers=(len(jobs) or 1) + 1) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([nvcc(), "-shared", "-cudart", "shared"] + ARCH + objs + ["-o", LIB])
    # drop-in source-compatibility check: user code written against the
    # reference's headers, compiled against ours and linked to the library
    if os.path.exists(dropin_src) and (force or _stale(dropin_lib, [dropin_src, LIB] + dropin_headers)):
        run([nvcc()] + NVCC_FLAGS + ARCH + ["-shared", "-cudart", "shared", dropin_src, "-o", dropin_lib,
             "-L" + HERE, "-lgallatin_gb300", "-Xlinker", "-rpath," + HERE])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
