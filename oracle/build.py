"""Build recipe for the CPU oracle and the reference-built checkers (test infrastructure only).

Under oracle/_build/ (this repository's own code, built wherever build() runs):

* ``libnlc_oracle.so``    -- the checker: oracle/nlc_oracle.c, -O2, no FP contraction, one thread;
* ``libnlc_oracle_mt.so`` -- the timed CPU baseline: the same source -Ofast with FMA contraction, as
  the reference builds its CPU code (CMakeLists.txt:62), OpenMP over copies.  Timing only;
* ``libref_gpu_host.so``  -- oracle/ref_shim/ref_gpu_host.cpp, the host side that launches the
  reference's own GPU kernels from the fatbins below (needs the CUDA toolkit; skipped without it).

Under oracle/_ref/, compiled in place from the reference's sources, only where they are present
(``NLC_REFERENCE_ROOT``, else a ``reference`` directory beside this repository):

* ``libref_symplectic.so`` -- the reference's Yoshida tables (common/symplectic.hpp), through
  oracle/ref_symplectic.cpp;
* ``nlchains-ref-cpu``      -- the reference's CPU program (the CMakeLists.txt:87-91 ``nlchains-cpu``
  target: common/main.cpp, results*.cpp and the three cpu-implementation files with their
  dispersion and eigensystem files), built -O2 without FP contraction, against the stand-ins for
  Boost, MPI, FFTW3 and Armadillo in oracle/ref_shim/ (an exact long-double DFT and a Jacobi
  eigensolver for the third-party arithmetic);
* ``nlchains-ref-cpu-oracle-math`` -- the same program whose FFT and eigensolver are the oracle's own
  (nlo_fft, nlo_eig_sym), for bit-for-bit comparisons of everything else;
* ``ref_gpu_n<N>.fatbin``   -- the reference's GPU sources (common/utilities_cuda.cu and the three model
  .cu files) compiled unmodified for sm_103a with optimized_chain_length = N, device code only,
  for N in REF_GPU_LENGTHS (the chain lengths of the benchmark configurations).

Nothing of the product imports, links or runs these files: only tests/, __graft_entry__.smoke() and
bench.py's baseline legs do.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "nlc_oracle.c")
REF_OUT = os.path.join(HERE, "_ref")
REF_SRC = os.path.join(HERE, "ref_symplectic.cpp")
SHIM = os.path.join(HERE, "ref_shim")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
REF_GPU_LENGTHS = (64, 128, 256)
REF_CPU_EXE = "nlchains-ref-cpu"
REF_CPU_EXE_ORACLE_MATH = "nlchains-ref-cpu-oracle-math"

# the nlchains-cpu target of the reference's CMakeLists.txt:87-91
REF_CPU_SOURCES = ["common/main.cpp", "common/results.cpp", "common/results_entropy.cpp",
                   "DNKG_FPUT_Toda/cpu-implementation/DNKG_FPUT_Toda.cpp", "DNKG_FPUT_Toda/dispersion.cpp",
                   "dDNKG/eigensystem.cpp", "dDNKG/cpu-implementation/dDNKG.cpp",
                   "DNLS/dispersion.cpp", "DNLS/cpu-implementation/DNLS.cpp"]
REF_GPU_SOURCES = ["common/utilities_cuda.cu", "DNKG_FPUT_Toda/DNKG_FPUT_Toda.cu", "dDNKG/dDNKG.cu", "DNLS/DNLS.cu"]

VARIANTS = {
    "libnlc_oracle.so": ["-O2"],
    "libnlc_oracle_mt.so": ["-Ofast", "-ffp-contract=fast", "-fopenmp"],
}


def reference_root():
    """The reference's source tree: $NLC_REFERENCE_ROOT, else ../reference beside the repository."""
    return os.environ.get("NLC_REFERENCE_ROOT") or os.path.join(os.path.dirname(REPO), "reference")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run_all(jobs, verbose, optional=False):
    """Run (cmd, target) pairs in parallel; each writes target + '.tmp', renamed on success."""
    procs = []
    for cmd, target in jobs:
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((subprocess.Popen(cmd), target))
    ok = True
    for p, target in procs:
        if p.wait() != 0:
            ok = False
            if not optional:
                raise RuntimeError("build failed: " + target)
            print("oracle build: " + os.path.basename(target) + " did not build", file=sys.stderr)
            continue
        os.replace(target + ".tmp", target)
    return ok


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "nlc_oracle.h"), __file__]
    jobs = []
    for name, flags in VARIANTS.items():
        target = os.path.join(OUT, name)
        if not _stale(target, deps):
            continue
        # the checker: -ffp-contract=off (gcc on aarch64 would otherwise fuse a*b+c, changing the
        # rounding); the baseline's own flags come after and override it
        jobs.append((["gcc", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                      *flags, "-o", target + ".tmp", SRC, "-lm"], target))
    host_src = os.path.join(SHIM, "ref_gpu_host.cpp")
    host = os.path.join(OUT, "libref_gpu_host.so")
    cuda_inc = os.path.join(CUDA_HOME, "include")
    if os.path.isdir(cuda_inc) and _stale(host, [host_src, __file__]):
        jobs.append((["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-I" + cuda_inc,
                      "-o", host + ".tmp", host_src, "-L" + os.path.join(CUDA_HOME, "lib64"),
                      "-L" + os.path.join(CUDA_HOME, "lib64", "stubs"), "-lcuda", "-lcudart", "-lcufft",
                      "-lcublas"], host))
    _run_all(jobs, verbose)
    return OUT


def build_ref(verbose=False):
    """Compile oracle/_ref from the reference sources; None where they are absent."""
    root = reference_root()
    header = os.path.join(root, "common", "symplectic.hpp")
    if not os.path.exists(header):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    build(verbose)
    jobs, optional = [], []
    target = os.path.join(REF_OUT, "libref_symplectic.so")
    if _stale(target, [REF_SRC, header, __file__]):
        jobs.append((["g++", "-std=c++17", "-fPIC", "-shared", "-O1", "-I", os.path.dirname(header),
                      "-o", target + ".tmp", REF_SRC], target))
    shim_files = [os.path.join(dp, f) for dp, _, fs in os.walk(SHIM) for f in fs]
    cpu_src = [os.path.join(root, s) for s in REF_CPU_SOURCES]
    common = ["-std=c++17", "-w", "-I" + SHIM, "-I" + root, "-I" + os.path.join(CUDA_HOME, "include"),
              "-include", os.path.join(SHIM, "ref_prelude.hpp")]
    # one rounding per C operator, no vector math library, no reassociation: the arithmetic the
    # oracle's reference order restates (the reference's own -Ofast build is the timing variant)
    strict = ["-O2", "-ffp-contract=off", "-fno-fast-math"]
    for exe, extra in ((REF_CPU_EXE, []),
                       (REF_CPU_EXE_ORACLE_MATH, ["-DREF_SHIM_ORACLE_MATH", "-L" + OUT, "-lnlc_oracle",
                                                  "-Wl,-rpath," + OUT])):
        target = os.path.join(REF_OUT, exe)
        if _stale(target, cpu_src + shim_files + [__file__, SRC]):
            jobs.append((["g++", *common, *strict, *cpu_src, os.path.join(SHIM, "ref_shim_impl.cpp"),
                          "-o", target + ".tmp", *extra, "-lm"], target))
    nvcc = os.path.join(CUDA_HOME, "bin", "nvcc")
    gpu_src = [os.path.join(root, s) for s in REF_GPU_SOURCES]
    cccl = os.path.join(CUDA_HOME, "include", "cccl")
    if os.path.exists(nvcc):
        for n in REF_GPU_LENGTHS:
            target = os.path.join(REF_OUT, f"ref_gpu_n{n}.fatbin")
            if _stale(target, gpu_src + shim_files + [__file__]):
                optional.append(([nvcc, "-std=c++17", "-fatbin", "-gencode", "arch=compute_103a,code=sm_103a",
                                  f"-Doptimized_chain_length={n}", "-w", "-I" + SHIM, "-I" + root, "-I" + cccl,
                                  "-include", os.path.join(SHIM, "ref_prelude.hpp"),
                                  os.path.join(SHIM, "ref_gpu_kernels.cu"), "-o", target + ".tmp"], target))
    if not _run_all(jobs, verbose, optional=True):   # the pins then skip
        print("oracle/_ref: part of the reference did not compile; its pins are skipped", file=sys.stderr)
    _run_all(optional, verbose, optional=True)
    return REF_OUT


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    build_ref(verbose="-v" in sys.argv)
