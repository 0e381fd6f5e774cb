"""Build libtdscha_gb300.so in-tree with nvcc for sm_103a.

    python -m tdscha_gb300.build        (or __graft_entry__.build())

Each .cu under csrc/ is compiled in parallel to an object, then linked into
one shared library with the static CUDA runtime.  The driver API entry
points (TMA descriptor encoding) are fetched at run time through
cudaGetDriverEntryPoint, so the library has no link-time libcuda dependency.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtdscha_gb300.so")
EXE_SRC = os.path.join(HERE, "exe", "tdscha_lanczos.cpp")
EXE = os.path.join(HERE, "tdscha-lanczos-gb300")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills"]


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _needs(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "tdscha_gb300.h"))
    jobs, objs = [], []
    for f in sources():
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f[:-3] + ".o")
        objs.append(obj)
        if force or _needs(obj, [src] + headers):
            jobs.append([NVCC] + ARCH + FLAGS + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _needs(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(tmp, LIB)
    build_exe(force)
    return LIB


def build_exe(force=False):
    """The input-file Lanczos program: host C++ linked against the library."""
    inc = os.path.join(os.path.dirname(HERE), "include")
    if not (force or _needs(EXE, [EXE_SRC, LIB, os.path.join(inc, "tdscha_gb300.h")])):
        return EXE
    tmp = EXE + ".tmp%d" % os.getpid()
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-I", inc, EXE_SRC, "-o", tmp,
           "-L", HERE, "-ltdscha_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("executable build failed: " + " ".join(cmd))
    os.replace(tmp, EXE)
    return EXE


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
