"""In-tree build of the engine: libnlchains_gb300.so and the `nlchains` executable.

Every CUDA translation unit is compiled for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``)
with ``-fmad=false`` (the kernels place every FMA explicitly) and host code with ``-ffp-contract=off``
(gcc on aarch64 would otherwise fuse a*b+c and change roundings).  Translation units compile in
parallel; outputs go next to this file (the library and the executable) and into _build/ (objects).
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnlchains_gb300.so")
EXE = os.path.join(HERE, "nlchains")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["nlc_real_toda.cu", "nlc_real_toda_short.cu", "nlc_real_dnkg.cu", "nlc_real_fput.cu", "nlc_real_ddnkg.cu",
              "nlc_diag.cu", "nlc_dnls.cu", "nlc_dnls_stencil.cu", "nlc_noalloc.cu", "nlc_energy.cu", "nlc_tc.cu"]
CPP_SOURCES = ["nlc_plan.cpp", "nlc_tables.cpp", "nlc_job.cpp", "nlc_server.cpp", "nlc_eig_device.cpp",
               "nlc_eig_host.cpp"]
# the host eigensolver's inner loops (products, rotations) want the vectoriser's full cost model
CPP_OPT = {"nlc_eig_host.cpp": "-O3"}
HEADERS = ["nlc_device.cuh", "nlc_real.cuh", "nlc_fft.cuh", "nlc_internal.h", "nlc_host.h", "nlc_fixed.h"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _cu_cmd(src, obj):
    return [NVCC, "-std=c++17", "-O3", *ARCH, "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
            "-I" + INCLUDE, "-c", src, "-o", obj]


def _cpp_cmd(src, obj):
    return ["g++", "-std=c++17", CPP_OPT.get(os.path.basename(src), "-O2"), "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
            "-I" + INCLUDE, "-I" + os.path.join(CUDA_HOME, "include"), "-c", src, "-o", obj]


def build(verbose=False):
    """Compile what is stale; return the path of the shared library."""
    os.makedirs(OBJ, exist_ok=True)
    common = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "nlchains.h"), __file__]
    jobs, objs = [], []
    for src in CU_SOURCES + CPP_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        if _newer(obj, [path] + common):
            cmd = _cu_cmd(path, obj) if src.endswith(".cu") else _cpp_cmd(path, obj)
            if verbose:
                print(" ".join(cmd), flush=True)
            jobs.append((subprocess.Popen(cmd), src))
    failed = [src for p, src in jobs if p.wait() != 0]
    if failed:
        raise RuntimeError("compilation failed: " + ", ".join(failed))
    if _newer(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [NVCC, "-shared", *ARCH, "-Xcompiler", "-fPIC", "-o", tmp, *objs, "-lpthread", "-ldl"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
        os.replace(tmp, LIB)
    cli_src = os.path.join(CSRC, "nlc_cli_main.cpp")
    if _newer(EXE, [LIB, cli_src]):
        cmd = ["g++", "-std=c++17", "-O2", "-I" + INCLUDE, cli_src, "-o", EXE + ".tmp", "-L" + HERE,
               "-lnlchains_gb300", "-Wl,-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
        os.replace(EXE + ".tmp", EXE)
    return LIB


def clean():
    shutil.rmtree(OBJ, ignore_errors=True)
    for p in (LIB, EXE):
        if os.path.exists(p):
            os.remove(p)


if __name__ == "__main__":
    if "clean" in sys.argv:
        clean()
    build(verbose="-v" in sys.argv)
