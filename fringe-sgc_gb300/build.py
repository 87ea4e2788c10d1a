"""Build libfsgc.so and the drop-in CLIs for sm_103a, in-tree.

Plain nvcc / g++ invocations run in parallel (no cmake): every .cu and .cpp
under csrc/ becomes an object, the objects link into _build/libfsgc.so, and
cli/*.cpp link against it as _build/fringePreprocess and _build/fringeCount.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INC = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(HERE, "csrc")]
LIB = os.path.join(OUT, "libfsgc.so")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    csrc = os.path.join(HERE, "csrc")
    headers = [os.path.join(csrc, f) for f in os.listdir(csrc) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "fsgc.h"))
    jobs = []
    objs = []
    for f in sorted(os.listdir(csrc)):
        src = os.path.join(csrc, f)
        obj = os.path.join(OUT, f + ".o")
        if f.endswith(".cu"):
            cmd = [NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr",
                   "-Xcompiler", "-fPIC,-fopenmp", "-Xptxas", "-v" if verbose else "-O3",
                   *INC, "-c", src, "-o", obj]
        elif f.endswith(".cpp"):
            cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-I" + os.path.join(CUDA, "include"),
                   *INC, "-c", src, "-o", obj]
        else:
            continue
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(cmd)
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    if _stale(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lgomp", "-lpthread"])
    clis = []
    for f in sorted(os.listdir(os.path.join(HERE, "cli"))):
        if not f.endswith(".cpp"):
            continue
        src = os.path.join(HERE, "cli", f)
        exe = os.path.join(OUT, f[:-4])
        if _stale(exe, [src, LIB]):
            clis.append(["g++", "-O2", "-std=c++17", *INC, src, "-o", exe, "-L" + OUT, "-lfsgc",
                         "-Wl,-rpath," + OUT])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(clis))) as ex:
        list(ex.map(_run, clis))
    if verbose:
        sys.stdout.write("".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
