"""Builds libptgpu.so in-tree: nvcc for the sm_103a kernels, g++ for the host
code, one shared library with the C ABI of include/ptgpu.h."""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libptgpu.so")

CU_SOURCES = ["lbvh.cu", "trace.cu", "wavefront.cu", "noalloc.cu", "batch.cu", "kd_gpu.cu", "ingest.cu",
              "image.cu"]
CPP_SOURCES = ["api.cpp", "kdtree.cpp", "loader.cpp", "batch.cpp", "server.cpp"]
HEADERS = ["device.cuh", "types.h", "lbvh.h", "lbvh_topo.cuh", "host.h", "devbuf.h", "ingest.h",
           "range_alloc.h", "step_policy.h"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no contraction, so float results round like the reference's
# OpenCL C; IEEE division and square root are nvcc's defaults.
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
                     "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-pthread"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found")


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, out_dir=None, lib_path=None, extra_nvcc=()):
    """Compiles into out_dir (default _build/) and links lib_path (default
    libptgpu.so); extra_nvcc adds nvcc flags (tuning experiments)."""
    out_dir = out_dir or OUT_DIR
    lib_path = lib_path or LIB
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(out_dir, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "ptgpu.h")]
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(out_dir, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append([nvcc] + NVCC_FLAGS + list(extra_nvcc) + ["-c", src, "-o", obj])
    for s in CPP_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(out_dir, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-I", os.path.join(cuda, "include"), "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("compile failed: %s" % cmd[-3])
    if force or jobs or not os.path.exists(lib_path):
        tmp = lib_path + ".tmp"
        cmd = [nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
