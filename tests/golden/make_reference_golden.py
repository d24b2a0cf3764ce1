"""Writes tests/golden/reference/*.npz by running the reference's own CPU program.

The program is the reference's ``nlchains-cpu`` (common/main.cpp with the five ``<model>-cpu``
subprograms of */cpu-implementation/*.cpp), compiled in place from the reference's sources by
oracle/build.py into oracle/_ref/ with stand-ins for its third-party libraries (oracle/ref_shim/):
Boost.ProgramOptions and a one-rank Boost.MPI, FFTW3 and Armadillo.  It is run twice per case:

* ``nlchains-ref-cpu``: the stand-in FFT is the exact discrete Fourier transform evaluated in long
  double and the stand-in eigensolver a long-double Jacobi -- FFTW's and LAPACK's results to an
  ulp or two;
* ``nlchains-ref-cpu-oracle-math``: the FFT and eigensolver are the oracle's own (nlo_fft,
  nlo_eig_sym), so that the oracle can be compared with the reference's arithmetic bit for bit.

Inputs are the seeded ensembles of nlchains_gb300/ic.py in the reference's -i file format, at the
shapes and parameters of the benchmark configurations (fewer copies).  Each fixture holds the input,
the parameters, and for both runs the state after `steps` steps (the reference's dump file), the
{t dt, WT, INF} entropy rows (the -entropy file) and the mode energies of every sample (the
-linenergies-<t> files).

Run from the repository root, where the reference's sources are present:
    python tests/golden/make_reference_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle.build as B  # noqa: E402
from nlchains_gb300 import ic  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference")

# name: (model, n, copies, dt, params, steps, batching, initial-state recipe)
CASES = {
    # FPUT-beta at the N = 64 benchmark configuration: energy density 0.1 over k = +-1..4
    "FPUT_n64_beta": ("FPUT", 64, 16, 0.1, dict(alpha=0.0, beta=1.0), 1000, 100,
                      dict(eps=0.1, kmax=4, include_zero=False)),
    # FPUT with a cubic term at an odd length (the reference's split kernel on the GPU)
    "FPUT_n37_alpha": ("FPUT", 37, 8, 0.1, dict(alpha=0.25, beta=1.0), 1000, 100,
                       dict(eps=0.1, kmax=3, include_zero=False)),
    # FPUT with every mode excited: no mode at rounding level, so the WT entropy is well conditioned
    "FPUT_n32_full": ("FPUT", 32, 8, 0.1, dict(alpha=0.25, beta=1.0), 1000, 100,
                      dict(eps=0.1, kmax=15, include_zero=False)),
    # DNKG and Toda at the N = 128 configuration: energy density 0.5 over the lowest 8% of modes
    "DNKG_n128": ("DNKG", 128, 8, 0.05, dict(m=1.0, beta=1.0), 1000, 100,
                  dict(eps=0.5, fraction=0.08, include_zero=True)),
    "Toda_n128": ("Toda", 128, 8, 0.05, dict(alpha=0.5), 1000, 100,
                  dict(eps=0.5, fraction=0.08, include_zero=False)),
    # DNKG below 32 sites (the reference's thread-per-chain kernel on the GPU)
    "DNKG_n12": ("DNKG", 12, 16, 0.05, dict(m=0.5, beta=1.0), 1000, 100,
                 dict(eps=0.5, kmax=5, include_zero=True)),
    # dDNKG at the N = 256 configuration: masses U[1, 3], energy 0.5 per site over 20 eigenmodes
    "dDNKG_n256": ("dDNKG", 256, 4, 0.05, dict(beta=1.0), 1000, 100, dict(eps=0.5, nmodes=20, mass_seed=777)),
    # DNLS at the N = 1024 configuration: norm density 1 over the lowest 10% of modes
    "DNLS_n1024": ("DNLS", 1024, 2, 0.01, dict(beta=1.0), 1000, 100,
                   dict(eps=1.0, fraction=0.1, include_zero=True)),
    "DNLS_n64": ("DNLS", 64, 4, 0.01, dict(beta=1.0), 1000, 100, dict(eps=1.0, fraction=0.1, include_zero=True)),
}
SEED = 2024


def initial_state(model, n, copies, params, recipe):
    """planar [copies][n][2] float64 (DNLS: re, im), as the benchmark's initial_state builds them."""
    if model == "dDNKG":
        masses = ic.masses_uniform(n, seed=recipe["mass_seed"])
        return ic.ddnkg_ensemble(masses, copies, recipe["eps"], recipe["nmodes"], seed=SEED), masses
    modes = ic.low_modes(n, recipe.get("fraction"), kmax=recipe.get("kmax"), include_zero=recipe["include_zero"])
    if model == "DNLS":
        psi = ic.dnls_ensemble(n, copies, recipe["eps"], modes, seed=SEED)
        return np.ascontiguousarray(psi).view(np.float64).reshape(copies, n, 2), None
    return ic.real_ensemble(n, copies, recipe["eps"], modes, m=params.get("m", 0.0), seed=SEED), None


def model_options(model, params, mfile):
    """The per-model options of DNKG_FPUT_Toda.cpp:26-45, dDNKG.cpp:31-34, DNLS.cpp:34-37."""
    if model == "DNKG":
        return ["-m", repr(params["m"]), "--beta", repr(params["beta"])]
    if model == "FPUT":
        return ["--alpha", repr(params["alpha"]), "--beta", repr(params["beta"])]
    if model == "Toda":
        return ["--alpha", repr(params["alpha"])]
    if model == "dDNKG":
        return ["-m", mfile, "--beta", repr(params["beta"])]
    return ["--beta", repr(params["beta"])]


def run_reference(exe, model, n, copies, dt, params, steps, batching, state, masses, work):
    init = os.path.join(work, "initial")
    state.astype(np.float64).tofile(init)
    mfile = os.path.join(work, "masses")
    if masses is not None:
        np.asarray(masses, dtype=np.float64).tofile(mfile)
    prefix = os.path.join(work, "run")
    cmd = [exe, model + "-cpu", "-i", init, "-n", str(n), "-c", str(copies), "--dt", repr(dt), "-b", str(batching),
           "-s", str(steps), "-p", prefix] + model_options(model, params, mfile)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)} failed:\n{r.stdout}\n{r.stderr}")
    out = {"state_out": np.fromfile(f"{prefix}-{steps}", dtype=np.float64).reshape(copies, n, 2),
           "entropy": np.fromfile(f"{prefix}-entropy", dtype=np.float64).reshape(-1, 3),
           "linenergies": np.stack([np.fromfile(f"{prefix}-linenergies-{t}", dtype=np.float64)
                                    for t in range(0, steps + 1, batching)])}
    if model == "dDNKG":
        out["omegas"] = np.fromfile(f"{prefix}-omegas", dtype=np.float64)
    return out


def make(name):
    model, n, copies, dt, params, steps, batching, recipe = CASES[name]
    state, masses = initial_state(model, n, copies, params, recipe)
    d = {"name": name, "model": model, "n": n, "copies": copies, "dt": dt, "steps": steps, "batching": batching,
         "m": params.get("m", 0.0), "alpha": params.get("alpha", 0.0), "beta": params.get("beta", 0.0),
         "state_in": state, "masses": masses if masses is not None else np.zeros(0)}
    for exe, suffix in ((B.REF_CPU_EXE, ""), (B.REF_CPU_EXE_ORACLE_MATH, "_om")):
        with tempfile.TemporaryDirectory() as work:
            res = run_reference(os.path.join(B.REF_OUT, exe), model, n, copies, dt, params, steps, batching, state,
                                masses, work)
        for k, v in res.items():
            d[k + suffix] = v
    return d


def main(names=None):
    if B.build_ref(verbose=False) is None:
        sys.exit("the reference's sources are not present (set NLC_REFERENCE_ROOT)")
    os.makedirs(OUT, exist_ok=True)
    for name in names or CASES:
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **make(name))
        print("wrote", name)


if __name__ == "__main__":
    main(sys.argv[1:])
