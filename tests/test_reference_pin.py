"""The oracle against the reference's own CPU program (tests/golden/reference, written by
tests/golden/make_reference_golden.py from the reference's sources compiled in place).

* With the oracle's FFT and eigensolver standing in for FFTW and LAPACK
  (``nlchains-ref-cpu-oracle-math``), the oracle's reference order reproduces the reference's program
  bit for bit: every sample's mode energies, every {t dt, WT, INF} entropy row and the final state,
  for all five models.
* With the exact discrete Fourier transform and a long-double Jacobi solver standing in for them
  (``nlchains-ref-cpu``): the real-model states are still bit-identical (no transform enters the
  integrator); mode energies and entropies agree to rounding; the DNLS state agrees to 1e-10 (the
  reference's |sin| = sqrt(1 - cos^2) rotation, DNLS/cpu-implementation/DNLS.cpp:85-95, turns an
  ulp of the transform into eps / angle^2 of the sine).
"""
import functools
import glob
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle as O
import oracle.build as B

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "reference", "*.npz")))


def load(path):
    d = dict(np.load(path))
    for k in ("name", "model"):
        d[k] = str(d[k])
    for k in ("n", "copies", "steps", "batching"):
        d[k] = int(d[k])
    for k in ("dt", "m", "alpha", "beta"):
        d[k] = float(d[k])
    return d


def params(d):
    return {"DNKG": dict(m=d["m"], beta=d["beta"]), "FPUT": dict(alpha=d["alpha"], beta=d["beta"]),
            "Toda": dict(alpha=d["alpha"]), "dDNKG": dict(beta=d["beta"]), "DNLS": dict(beta=d["beta"])}[d["model"]]


def oracle_model(d, order=O.ORDER_REFERENCE):
    return O.Model(d["model"], d["n"], d["copies"], d["dt"], masses=d["masses"] if d["model"] == "dDNKG" else None,
                   order=order, **params(d))


@functools.lru_cache(maxsize=None)
def oracle_run_cached(path):
    return oracle_run(load(path))


def oracle_run(d):
    """The oracle's reference order over the fixture's run: per-sample mode energies, entropy rows, final state."""
    mdl = oracle_model(d)
    eig = O.eigensystem(d["n"], mdl.mp2) if d["model"] == "dDNKG" else None
    st = d["state_in"].copy()
    lins, rows = [], []
    samples = d["steps"] // d["batching"] + 1
    for s in range(samples):
        lin = O.linenergies(mdl, st, eig)
        wt, inf = O.entropies(lin, O.a0is0(mdl))
        lins.append(lin)
        rows.append((s * d["batching"] * d["dt"], wt, inf))
        if s + 1 < samples:
            st = O.advance(mdl, st, d["batching"], d["batching"], order=O.ORDER_REFERENCE).reshape(st.shape)
    return np.array(lins), np.array(rows), st


def well_conditioned(lin):
    """WT = -sum log e_k is ill-conditioned where a mode sits at rounding level (an unexcited mode of
    a low-mode initial state): compare it only where every mode carries energy."""
    return lin[1:].min() > 1e-8 * lin.max()


def test_fixtures_present():
    assert len(FIXTURES) >= 9
    models = {load(p)["model"] for p in FIXTURES}
    assert models == {"DNKG", "FPUT", "Toda", "dDNKG", "DNLS"}


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_is_the_reference_program_bit_for_bit(path):
    d = load(path)
    lins, rows, st = oracle_run_cached(path)
    assert np.array_equal(st, d["state_out_om"]), "final state differs from the reference program's dump"
    assert np.array_equal(lins, d["linenergies_om"]), "mode energies differ from the reference program's"
    assert np.array_equal(rows, d["entropy_om"]), "entropy rows differ from the reference program's"


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_the_reference_program_with_exact_transforms(path):
    d = load(path)
    lins, rows, st = oracle_run_cached(path)
    if d["model"] == "DNLS":
        assert np.abs(st - d["state_out"]).max() <= 1e-10 * np.abs(d["state_out"]).max()
    else:
        assert np.array_equal(st, d["state_out"])
    for s in range(len(lins)):
        ref = d["linenergies"][s]
        assert np.abs(lins[s] - ref).max() <= 1e-10 * ref.max(), f"sample {s}"
        assert rows[s][0] == d["entropy"][s][0]
        assert abs(rows[s][2] - d["entropy"][s][2]) <= 1e-10 * abs(d["entropy"][s][2]), f"INF, sample {s}"
        if well_conditioned(ref):
            assert abs(rows[s][1] - d["entropy"][s][1]) <= 1e-10 * max(1.0, abs(d["entropy"][s][1])), f"WT, sample {s}"


def test_every_fixture_reaches_a_well_conditioned_sample():
    """Each run ends with energy in every mode, so its last samples also pin the WT entropy."""
    for p in FIXTURES:
        d = load(p)
        assert well_conditioned(d["linenergies"][-1]), d["name"]


def test_ddnkg_frequencies_are_the_reference_eigensystem():
    d = load(os.path.join(HERE, "golden", "reference", "dDNKG_n256.npz"))
    om, _ = O.eigensystem(d["n"], d["masses"] + 2)
    assert np.abs(om - d["omegas"]).max() <= 1e-13 * om.max()
    assert np.array_equal(om, d["omegas_om"])


def _reference_program(exe):
    path = os.path.join(B.REF_OUT, exe)
    if not os.path.exists(os.path.join(B.reference_root(), "common", "main.cpp")):
        pytest.skip("the reference's sources are not on this machine")
    B.build_ref()
    if not os.path.exists(path):
        pytest.skip("the reference's CPU program did not build here")
    return path


def test_fixture_is_current():
    """Re-run the reference's program on one fixture's input: the committed outputs are what it writes."""
    import importlib.util
    exe = _reference_program(B.REF_CPU_EXE)
    spec = importlib.util.spec_from_file_location("mrg", os.path.join(HERE, "golden", "make_reference_golden.py"))
    mrg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mrg)
    d = load(os.path.join(HERE, "golden", "reference", "DNKG_n12.npz"))
    with tempfile.TemporaryDirectory() as work:
        res = mrg.run_reference(exe, d["model"], d["n"], d["copies"], d["dt"], params(d), d["steps"],
                                d["batching"], d["state_in"], None, work)
    assert np.array_equal(res["state_out"], d["state_out"])
    assert np.array_equal(res["entropy"], d["entropy"])
    assert np.array_equal(res["linenergies"], d["linenergies"])


def test_reference_program_validates_its_command_line():
    """The stand-in option parser keeps the reference's validation (common/main.cpp:82-103)."""
    exe = _reference_program(B.REF_CPU_EXE)
    with tempfile.TemporaryDirectory() as work:
        init = os.path.join(work, "init")
        np.zeros((2, 8, 2)).tofile(init)
        base = [exe, "DNKG-cpu", "-i", init, "-n", "8", "-c", "2", "--dt", "0.1", "-p", os.path.join(work, "x"),
                "-m", "1", "--beta", "1"]
        r = subprocess.run(base + ["-b", "10", "-s", "15"], capture_output=True, text=True)
        assert r.returncode == 1 and "--steps must be a multiple of --kernel_batching" in r.stderr
        r = subprocess.run(base[:-4] + ["-b", "10", "-s", "10"], capture_output=True, text=True)
        assert r.returncode == 1 and "required" in r.stderr
        r = subprocess.run(base + ["-b", "10", "-s", "10"], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
