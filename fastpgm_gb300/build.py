"""In-tree build of the engine library and command line (sm_103a only).

Outputs (git-ignored):
  fastpgm_gb300/lib/libfastpgm_gb300.so   CUDA kernels + C ABI + C++ drop-in classes
  fastpgm_gb300/bin/fastpgm               `-j 0 -m 0` command line
Object files go to fastpgm_gb300/_build/.  Translation units compile in parallel;
a unit is rebuilt only when its source or any header is newer than its object.
"""
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libfastpgm_gb300.so")
CLI = os.path.join(BINDIR, "fastpgm")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    for c in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _headers():
    return glob.glob(os.path.join(CSRC, "**", "*.h*"), recursive=True) + glob.glob(
        os.path.join(ROOT, "include", "*.h"))


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(f) > t for f in [src] + _headers())


def build(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
    units = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        units.append((src, obj, [nvcc()] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC"] + inc
                      + ["-c", src, "-o", obj]))
    host = [os.path.join(CSRC, "datagen.cpp")] + sorted(glob.glob(os.path.join(CSRC, "host", "*.cpp")))
    for src in host:
        if src.endswith("main.cpp"):
            continue
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        extra = ["-ffp-contract=off", "-fopenmp"] if src.endswith("datagen.cpp") else ["-fopenmp"]
        units.append((src, obj, ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wextra"] + extra + inc
                      + ["-I" + cuda_inc, "-c", src, "-o", obj]))
    procs = []
    for src, obj, cmd in units:
        if _stale(obj, src):
            if verbose:
                print(" ".join(cmd))
            procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errs = []
    for src, p in procs:
        out = p.communicate()[0].decode()
        if p.returncode != 0:
            errs.append("%s:\n%s" % (src, out))
        elif verbose and out.strip():
            print(out)
    if errs:
        raise RuntimeError("build failed:\n" + "\n".join(errs))
    objs = [u[1] for u in units]
    if procs or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"]
        subprocess.check_call(cmd)
    main_src = os.path.join(CSRC, "host", "main.cpp")
    if procs or not os.path.exists(CLI) or os.path.getmtime(main_src) > os.path.getmtime(CLI):
        cmd = ["g++", "-O2", "-std=c++17"] + inc + ["-I" + cuda_inc, main_src, "-o", CLI, "-L" + LIBDIR,
                                                     "-lfastpgm_gb300", "-Wl,-rpath,$ORIGIN/../lib"]
        subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
