"""In-tree build of libmilc_ks_gb300.so (CUDA kernels for sm_103a + C host code).

The library is a plain C-ABI shared object: nvcc compiles every ``csrc/*.cu``
for ``sm_103a`` only, gcc compiles ``csrc/*.c``, and nvcc links them with
``-shared``.  Translation units compile in parallel; objects are rebuilt
only when a source or header is newer.
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJDIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmilc_ks_gb300.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-fopenmp", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
# extra nvcc flags for measurement builds (e.g. "-DMKS_NBR_LEX=0"); objects
# are rebuilt when the flags change
EXTRA_NVFLAGS = os.environ.get("MKS_NVFLAGS", "").split()
CFLAGS = ["-O2", "-g", "-std=gnu99", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function",
          "-I" + os.path.join(ROOT, "include")]


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + deps)


def _compile(job):
    cmd, obj = job
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed for %s:\n%s\n%s" % (obj, " ".join(cmd), r.stderr[-6000:]))
    return obj


def build(verbose=False, extra_nvflags=()):
    """Compile the library if needed and return its path."""
    os.makedirs(OBJDIR, exist_ok=True)
    deps = _headers()
    flags = NVFLAGS + EXTRA_NVFLAGS + list(extra_nvflags)
    stamp = os.path.join(OBJDIR, "nvflags")
    old = open(stamp).read() if os.path.exists(stamp) else None
    if old != " ".join(flags):
        with open(stamp, "w") as f:
            f.write(" ".join(flags))
    jobs, objs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src, deps + [stamp]):
            jobs.append(([NVCC] + ARCH + flags + ["-c", src, "-o", obj], obj))
    for src in sorted(glob.glob(os.path.join(CSRC, "*.c"))):
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            jobs.append((["gcc"] + CFLAGS + ["-c", src, "-o", obj], obj))
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for o in ex.map(_compile, jobs):
                if verbose:
                    print("compiled", os.path.relpath(o, ROOT), file=sys.stderr)
    if jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-6000:]))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
