"""Build recipe of libgala.so and the two CLIs (gala_main, gala_preprocess).

nvcc compiles the CUDA translation units for sm_103a only
(-gencode arch=compute_103a,code=sm_103a); host code is C++17.  All FP64
code is built without fused multiply-add contraction (--fmad=false for
device code, -ffp-contract=off for host code) so the engine's gain and
modularity arithmetic rounds exactly as written.  Outputs go to
gala-mg_gb300/_build/ (git-ignored).  Translation units compile in parallel;
an output newer than all its inputs is not rebuilt.

    python gala-mg_gb300/build.py          # build
    python gala-mg_gb300/build.py --force  # rebuild everything
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
INC = os.path.join(os.path.dirname(PKG), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_UNITS = ["phase1.cu", "contract.cu", "engine.cu", "modularity_static.cu", "proposal.cu", "batch.cu", "refine.cu",
            "batch_cta.cu", "update_push.cu"]
CPP_UNITS = ["graph_host.cpp"]
CLIS = ["gala_main.cpp", "gala_preprocess.cpp"]
HEADERS = ["common.cuh", "scan.cuh", "walk.cuh", "internal.h", "binlimits.h"]


def _nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _stale(out, ins):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(i) > t for i in ins)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def lib_path():
    return os.path.join(OUT, "libgala.so")


def build(force=False, verbose=False, extra_nvcc=()):
    os.makedirs(OUT, exist_ok=True)
    hdrs = [os.path.join(SRC, h) for h in HEADERS] + [os.path.join(INC, "gala.h")]
    jobs = []
    objs = []
    nvcc = _nvcc()
    cuda_inc = os.path.join(_cuda_home(), "include")
    for u in CU_UNITS:
        src = os.path.join(SRC, u)
        obj = os.path.join(OUT, u + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs + [__file__]):
            jobs.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "--fmad=false", "-Xcompiler",
                         "-fPIC,-ffp-contract=off", "-I", INC, *extra_nvcc, "-c", src, "-o", obj])
    for u in CPP_UNITS:
        src = os.path.join(SRC, u)
        obj = os.path.join(OUT, u + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs + [__file__]):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I", INC, "-I",
                         cuda_inc, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    lib = lib_path()
    if force or jobs or _stale(lib, objs):
        _run([nvcc, *ARCH, "-shared", "-o", lib, *objs, "-lpthread"])
    for c in CLIS:
        exe = os.path.join(OUT, c[:-4])
        src = os.path.join(SRC, c)
        if force or _stale(exe, [src, lib, os.path.join(INC, "gala.h")]):
            _run(["g++", "-O2", "-std=c++17", "-I", INC, src, "-o", exe, "-L", OUT, "-lgala",
                  "-Wl,-rpath,$ORIGIN"])
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print("built", lib_path())
