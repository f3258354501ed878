"""Builds rayt_gb300/_lib/librayt_gb300.so (the product library) and
oracle/_build/librayt_oracle.so (the CPU oracle used by tests and the CPU
baseline).  Every CUDA file is compiled for sm_103a only."""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "rayt_gb300", "csrc")
LIB_DIR = os.path.join(ROOT, "rayt_gb300", "_lib")
ORACLE_DIR = os.path.join(ROOT, "oracle", "_build")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# FP32 traversal must not fuse or approximate: it is compared bit for bit with
# the reference's operation order.
CU_FLAGS = ["-O3", "-std=c++17", "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
            "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread"]

CU_SOURCES = ["trace.cu", "sort.cu", "upload.cu", "unique_noalloc.cu"]
CXX_SOURCES = ["util.cpp", "tree.cpp", "cache.cpp", "renderer.cpp", "server.cpp", "prims.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force=False):
    os.makedirs(os.path.join(LIB_DIR, "obj"), exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    headers.append(os.path.join(ROOT, "include", "rayt_gb300.h"))
    jobs = []
    objs = []
    for f in CU_SOURCES + CXX_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(LIB_DIR, "obj", f + ".o")
        objs.append(obj)
        if not force and not _newer(obj, [src, __file__] + headers):
            continue
        if f.endswith(".cu"):
            jobs.append([NVCC] + ARCH + CU_FLAGS + ["-c", src, "-o", obj])
        else:
            jobs.append(["g++"] + CXX_FLAGS + ["-I", os.path.join(CUDA_HOME, "include"), "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        list(ex.map(_run, jobs))
    lib = os.path.join(LIB_DIR, "librayt_gb300.so")
    if force or jobs or not os.path.exists(lib):
        _run([NVCC] + ARCH + ["-shared", "-o", lib] + objs + ["-lpthread"])
    return lib


def build_oracle(force=False):
    os.makedirs(ORACLE_DIR, exist_ok=True)
    src = os.path.join(ROOT, "oracle", "rayt_oracle.cpp")
    lib = os.path.join(ORACLE_DIR, "librayt_oracle.so")
    if force or _newer(lib, [src]):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared", "-o", lib, src])
    return lib


def build_reference_harness():
    """Compiles the reference's own code into oracle/_ref when RAYT_REFERENCE
    names a reference checkout (the directory holding rayt/); skipped
    otherwise.  Only the golden-fixture generator uses it."""
    ref = os.environ.get("RAYT_REFERENCE")
    if not ref or not os.path.isdir(os.path.join(ref, "rayt")):
        return None
    _run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")])
    return os.path.join(ROOT, "oracle", "_ref", "librayt_ref.so")


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_library(force))
    print(build_oracle(force))
