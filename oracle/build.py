"""Build recipe for the CPU oracle (test infrastructure only).

Two shared objects are produced under oracle/_build/ from oracle/nlc_oracle.c:

* ``libnlc_oracle.so``  -- the checker: -O2, no FP contraction, single thread;
* ``libnlc_oracle_mt.so`` -- the timed CPU baseline: -Ofast with FMA contraction, as the reference
  builds its CPU code (CMakeLists.txt:62), OpenMP over copies.  Timing only: its arithmetic is not
  the checker's.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use these libraries.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "nlc_oracle.c")

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


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
