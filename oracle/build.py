"""Build recipe for the CPU oracle (test infrastructure only).

Two shared objects are produced under oracle/_build/ from oracle/nlc_oracle.c:

* ``libnlc_oracle.so``  -- the checker: -O2, no FP contraction, single thread;
* ``libnlc_oracle_mt.so`` -- the timed CPU baseline: -Ofast with FMA contraction, as the reference
  builds its CPU code (CMakeLists.txt:62), OpenMP over copies.  Timing only: its arithmetic is not
  the checker's.

and, where the reference sources are present, one under oracle/_ref/:

* ``libref_symplectic.so`` -- the reference's own Yoshida tables (common/symplectic.hpp, compiled in
  place by oracle/ref_symplectic.cpp), which the tests pin the oracle's tables to.  The rest of the
  reference's path needs Boost, MPI, FFTW3 and Armadillo and is not built.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use these libraries.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "nlc_oracle.c")
REF_OUT = os.path.join(HERE, "_ref")
REF_SRC = os.path.join(HERE, "ref_symplectic.cpp")
REFERENCE_ROOT = os.environ.get("NLC_REFERENCE_ROOT", "/root/reference")

VARIANTS = {
    "libnlc_oracle.so": ["-O2"],
    "libnlc_oracle_mt.so": ["-Ofast", "-ffp-contract=fast", "-fopenmp"],
}


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "nlc_oracle.h"), __file__]
    procs = []
    for name, flags in VARIANTS.items():
        target = os.path.join(OUT, name)
        if not _stale(target, deps):
            continue
        # the checker: -ffp-contract=off (gcc on aarch64 would otherwise fuse a*b+c, changing the
        # rounding); the baseline's own flags come after and override it
        cmd = ["gcc", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
               *flags, "-o", target + ".tmp", SRC, "-lm"]
        if verbose:
            print(" ".join(cmd))
        procs.append((subprocess.Popen(cmd), target))
    for p, target in procs:
        if p.wait() != 0:
            raise RuntimeError("oracle build failed: " + target)
        os.replace(target + ".tmp", target)
    return OUT


def build_ref(verbose=False):
    """Compile oracle/_ref from the reference sources; None where they are absent."""
    header = os.path.join(REFERENCE_ROOT, "common", "symplectic.hpp")
    if not os.path.exists(header):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    target = os.path.join(REF_OUT, "libref_symplectic.so")
    if _stale(target, [REF_SRC, header, __file__]):
        cmd = ["g++", "-std=c++17", "-fPIC", "-shared", "-O1", "-I", os.path.dirname(header),
               "-o", target + ".tmp", REF_SRC]
        if verbose:
            print(" ".join(cmd))
        if subprocess.run(cmd).returncode != 0:   # optional: the pin test then skips
            print("oracle/_ref: the reference header did not compile; its pin is skipped", file=sys.stderr)
            return None
        os.replace(target + ".tmp", target)
    return REF_OUT


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    build_ref(verbose="-v" in sys.argv)
