"""Build libsdegpu.so (sm_103a) in-tree: sde_gb300/_lib/libsdegpu.so.

Each .cu translation unit is compiled in parallel with nvcc for
-gencode arch=compute_103a,code=sm_103a, then linked into one shared library against the
static CUDA runtime.  The driver API (cuTensorMapEncodeTiled) is resolved at run time through
cudaGetDriverEntryPointByVersion, so the library loads on machines without a GPU driver.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libsdegpu.so")
SOURCES = ["api.cu", "sort.cu", "weights.cu", "plan.cu", "grid.cu", "fft.cu", "clean.cu", "batch.cu", "jobs.cu", "uvfits.cu", "clark.cu", "dft.cu", "model.cu", "box.cu", "slowz.cu", "uruwt.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off", "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _stale(lib, deps):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, ptxas_info=False):
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(SRC, s) for s in SOURCES] + [
        os.path.join(SRC, "common.cuh"), os.path.join(HERE, "..", "include", "sde_gpu.h"),
        os.path.abspath(__file__)]
    if not force and not _stale(LIB, deps):
        return LIB
    nv = nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_one(src):
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        cmd = [nv, *ARCH, *FLAGS, *extra, "-c", os.path.join(SRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose or ptxas_info:
        for obj, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-ldl", "-lpthread", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_info="-v" in sys.argv))
