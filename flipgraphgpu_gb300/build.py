"""Builds libflipgraph.so (CUDA, sm_103a) and the three CLI executables.

    python -m flipgraphgpu_gb300.build [--clean]

Each .cu translation unit under csrc/ is compiled in parallel with
`nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo`, linked into
flipgraphgpu_gb300/_lib/<machine>/libflipgraph.so; the C++ CLIs under cli/
link against it with an rpath.  No cmake, no torch extension machinery.
"""
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
CLI = os.path.join(PKG, "cli")
OUT = os.path.join(PKG, "_lib", platform.machine())
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                  "-I", os.path.join(ROOT, "include"), "-I", CSRC]
CXXFLAGS = ["-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include")]


def lib_path():
    return os.path.join(OUT, "libflipgraph.so")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}")
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, extra=()):
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "flipgraph.h"))
    units = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    jobs = []
    for u in units:
        src = os.path.join(CSRC, u)
        obj = os.path.join(OUT, "obj", u[:-3] + ".o")
        if _stale(obj, [src] + headers):
            jobs.append([NVCC] + NVFLAGS + list(extra) + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    objs = [os.path.join(OUT, "obj", u[:-3] + ".o") for u in units]
    lib = lib_path()
    if _stale(lib, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])
    # CLI executables (host C++ only; they reach CUDA through the C-ABI).
    if os.path.isdir(CLI):
        common = sorted(os.path.join(CLI, f) for f in os.listdir(CLI) if f.endswith(".cpp") and not f.startswith("main_"))
        cheaders = [os.path.join(CLI, f) for f in os.listdir(CLI) if f.endswith(".h")]
        cjobs = []
        for main in sorted(f for f in os.listdir(CLI) if f.startswith("main_") and f.endswith(".cpp")):
            exe = os.path.join(OUT, main[len("main_"):-4])
            srcs = [os.path.join(CLI, main)] + common
            if _stale(exe, srcs + cheaders + [lib]):
                cjobs.append(["g++"] + CXXFLAGS + srcs + ["-o", exe, "-L", OUT, "-lflipgraph",
                                                         "-Wl,-rpath," + OUT])
        with cf.ThreadPoolExecutor(max(1, len(cjobs))) as ex:
            list(ex.map(_run, cjobs))
    return lib


if __name__ == "__main__":
    if "--clean" in sys.argv:
        shutil.rmtree(OUT, ignore_errors=True)
    print(build(verbose="-v" in sys.argv, extra=["-Xptxas", "-v"] if "-v" in sys.argv else ()))
