"""Build libcaustics_gb300.so in-tree with nvcc for sm_103a (GB300).

Each translation unit in csrc/ is compiled in parallel, then linked into
caustics_gb300/libcaustics_gb300.so (the C ABI of include/caustics_gb300.h).
csrc/bench/ holds the benchmark's measurement probe, linked on its own into
caustics_gb300/libcgb_bench.so so that the product library carries none of it.
Rebuilds only what changed.

    python -m caustics_gb300.build [-v]
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcaustics_gb300.so")
BENCH_LIB = os.path.join(HERE, "libcgb_bench.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build caustics_gb300")
    return cand


def _cuda_lib_dir(nvcc):
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        d = os.path.join(root, sub)
        if os.path.exists(os.path.join(d, "libcudart.so")) or glob.glob(os.path.join(d, "libcudart.so.*")):
            return d
    return os.path.join(root, "lib64")


def _deps_mtime():
    files = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
    files.append(os.path.join(os.path.dirname(HERE), "include", "caustics_gb300.h"))
    return max(os.path.getmtime(f) for f in files if os.path.exists(f))


def build(verbose=False, jobs=None):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    hdr_t = _deps_mtime()
    todo = []
    libs = []
    for lib, sources in ((LIB, sorted(glob.glob(os.path.join(CSRC, "*.cu")))),
                         (BENCH_LIB, sorted(glob.glob(os.path.join(CSRC, "bench", "*.cu"))))):
        objs = []
        for src in sources:
            obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
            objs.append(obj)
            if not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_t):
                todo.append((src, obj))
        libs.append((lib, objs))

    def compile_one(job):
        src, obj = job
        cmd = [nvcc] + ARCH + FLAGS + ["-c", src, "-o", obj + ".tmp"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        os.replace(obj + ".tmp", obj)
        return src

    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for done in ex.map(compile_one, todo):
                if verbose:
                    print("compiled", os.path.basename(done), flush=True)
    libdir = _cuda_lib_dir(nvcc)
    for lib, objs in libs:
        if not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
            cmd = [nvcc] + ARCH + ["-shared", "--cudart", "shared", "-o", lib + ".tmp"] + objs + [
                "-Xlinker", f"-rpath,{libdir}"]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link of {os.path.basename(lib)} failed:\n{r.stdout}\n{r.stderr}")
            os.replace(lib + ".tmp", lib)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
