"""Build libvmck.so (the CUDA kernels + C ABI) in-tree for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled in parallel with nvcc, then
linked against cuBLAS / cuSOLVER into ``netket_gb300/_lib/libvmck.so``.
Nothing is installed outside the repository.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libvmck.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-Xptxas", "-O3"]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_lib_dir(nvcc):
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    for d in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"),
              os.path.join("targets", "x86_64-linux", "lib")):
        p = os.path.join(root, d)
        if os.path.exists(os.path.join(p, "libcublas.so")):
            return p
    return os.path.join(root, "lib64")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, extra_flags=()):
    nvcc = nvcc_path()
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "vmck.h"))
    objs, jobs = [], []
    for src in sources():
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src[:-3] + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra_flags, "-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, flush=True)

    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB) or _newer(LIB, objs):
        libdir = cuda_lib_dir(nvcc)
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, f"-L{libdir}", "-lcublas", "-lcusolver",
               "-Xlinker", f"-rpath={libdir}"]
        run(cmd)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
