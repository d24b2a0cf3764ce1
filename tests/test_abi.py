"""The C ABI library: it builds, loads, and exports every symbol include/nlchains.h declares; the
command line, the plan constructor and the no-alloc entry point reject invalid arguments before
touching a GPU, and the host entropies keep their error behaviour (CPU only)."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            text = open(os.path.join(ROOT, "include", name)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            syms |= set(re.findall(r"\b(nlc_[a-z0-9_]+)\s*\(", text))
    return syms


def test_library_exports_every_declared_symbol(engine):
    lib = engine.lib()
    missing = [s for s in sorted(declared_symbols()) if not hasattr(lib, s)]
    assert not missing, missing
    assert set(engine.EXPORTS) == declared_symbols()
    assert engine.lib().nlc_version().startswith(b"nlchains-gb300")


@pytest.mark.parametrize("args,needle", [
    (["FPUT", "-n", "64"], "is required"),
    (["FPUT", "-i", "x", "-n", "64", "-c", "4", "--dt", "0.1", "-b", "10", "-s", "15", "-p", "o", "--alpha", "0",
      "--beta", "1"], "--steps must be a multiple of --kernel_batching"),
    (["FPUT", "-i", "x", "-n", "1", "-c", "4", "--dt", "0.1", "-b", "10", "-p", "o", "--alpha", "0", "--beta", "1"],
     "--chain_length must be >= 2"),
    (["FPUT", "-i", "x", "-n", "8", "-c", "4", "--dt", "0.1", "-b", "10", "--dump_interval", "15", "-p", "o",
      "--alpha", "0", "--beta", "1"], "--dump_interval must be a multiple of --kernel_batching"),
    (["FPUT", "-i", "x", "-n", "8", "-c", "4", "--dt", "0.1", "-b", "10", "-s", "10", "-o", "10", "-p", "o",
      "--alpha", "0", "--beta", "1"], "--time_offset must be less than --steps"),
    (["Toda", "-i", "x", "-n", "8", "-c", "4", "--dt", "0.1", "-b", "10", "-p", "o"], "'--alpha' is required"),
    (["FPUT", "-i", "missing-file", "-n", "8", "-c", "4", "--dt", "0.1", "-b", "10", "-p", "o", "--alpha", "0",
      "--beta", "1"], "could not read initial state"),
    (["FPUT-cpu"], "not part of this engine"),
    (["NOPE"], "valid program"),
    (["DNKG", "--bogus", "1"], "unrecognised option"),
])
def test_cli_rejects_invalid_arguments(engine, tmp_path, args, needle):
    r = subprocess.run([engine.EXECUTABLE_PATH, *args], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert needle in r.stderr


COMMON = ["-n", "8", "-c", "4", "--dt", "0.1", "-b", "10", "-p", "o"]


@pytest.mark.parametrize("args,needle", [
    (["dDNKG", "-i", "init", *COMMON, "-m", "masses5", "--beta", "1"], "could not read m file (masses5)"),
    (["dDNKG", "-i", "init", *COMMON, "-m", "missing", "--beta", "1"], "could not read m file (missing)"),
    (["FPUT", "-i", "init", *COMMON, "--alpha", "0", "--beta", "1", "--entropymask", "mask3"],
     "could not read entropy mask file (mask3)"),
    (["FPUT", "-i", "init3", *COMMON, "--alpha", "0", "--beta", "1"], "could not read initial state (init3)"),
    (["FPUT", "-i", "init", "-n", "8", "-c", "4", "--dt", "-1", "-b", "10", "-p", "o", "--alpha", "0", "--beta", "1"],
     "must be positive numbers"),
    (["FPUT", "-i", "init", "-n", "8", "-c", "4", "--dt", "0.1", "-b", "0", "-p", "o", "--alpha", "0", "--beta", "1"],
     "must be positive numbers"),
    (["DNKG", "-i", "init", *COMMON, "-m", "abc", "--beta", "1"], "the argument ('abc') for option '--m' is invalid"),
])
def test_cli_rejects_invalid_files_and_values(engine, tmp_path, args, needle):
    """Files of the wrong size (masses of 5 sites for 8, a 3-byte mask, 3 of the 4 chains) and
    non-numeric or non-positive values are refused before the GPU is touched, with exit code 1."""
    np.zeros((4, 8, 2)).tofile(tmp_path / "init")
    np.zeros((3, 8, 2)).tofile(tmp_path / "init3")
    np.ones(5).tofile(tmp_path / "masses5")
    np.ones(3, dtype=np.uint8).tofile(tmp_path / "mask3")
    r = subprocess.run([engine.EXECUTABLE_PATH, *args], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert needle in r.stderr


def test_cli_usage_without_options(engine):
    r = subprocess.run([engine.EXECUTABLE_PATH, "DNLS"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "--beta" in r.stdout and "--no_linear_callback" in r.stdout
    r = subprocess.run([engine.EXECUTABLE_PATH], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "subprogram" in r.stdout


@pytest.mark.parametrize("kw,needle", [
    (dict(model=9, chain_length=8, copies=4, dt=0.1), "unknown model id"),
    (dict(model="DNKG", chain_length=1, copies=4, dt=0.1), "--chain_length must be >= 2"),
    (dict(model="DNKG", chain_length=65536, copies=4, dt=0.1), "fit 16 bits"),
    (dict(model="FPUT", chain_length=8, copies=0, dt=0.1), "--copies must be a positive number"),
    (dict(model="Toda", chain_length=8, copies=4, dt=0.0), "--dt must be a positive number"),
    (dict(model="DNLS", chain_length=8, copies=4, dt=float("nan")), "--dt must be a positive number"),
    (dict(model="dDNKG", chain_length=8, copies=4, dt=0.1), "needs the per-site masses"),
    (dict(model="DNKG", chain_length=65535, copies=1 << 25, dt=0.1), "too large"),
])
def test_plan_rejects_invalid_models_before_any_device_call(engine, kw, needle):
    with pytest.raises(engine.NlcError) as e:
        engine.Plan(engine.Model(**kw))
    assert e.value.code == engine.EINVAL and needle in str(e.value)
    assert needle in engine.last_error()


@pytest.mark.parametrize("args,needle", [
    ((3, 64, 8, 0.0, 16, None, 16, None, None), "model must be DNKG, FPUT, Toda or DNLS"),
    ((0, 64, 8, 0.0, None, None, 16, None, None), "NULL state or output"),
    ((0, 1, 8, 0.0, 16, None, 16, None, None), "chain_length >= 2 and copies > 0"),
    ((0, 64, 0, 0.0, 16, None, 16, None, None), "chain_length >= 2 and copies > 0"),
    ((4, 4097, 8, 0.0, 16, None, 16, None, None), "does not fit the 4 MiB static scratch"),
])
def test_noalloc_rejects_invalid_arguments_before_any_device_call(engine, args, needle):
    """The pointers given are never dereferenced: every case returns at an argument check that runs
    before the first CUDA call."""
    assert engine.lib().nlc_linenergies_noalloc(*args) == engine.EINVAL
    assert needle in engine.last_error()


@pytest.mark.parametrize("n", [1021, 4093, 2 * 67, 3 * 1009])
def test_noalloc_rejects_large_prime_factors_before_any_device_call(engine, n):
    """A prime factor above 61 would be one thread's direct transform per chain: refused up front."""
    assert engine.lib().nlc_linenergies_noalloc(0, n, 8, 0.0, 16, None, 16, None, None) == engine.EUNSUPPORTED
    assert "prime factor above 61" in engine.last_error()


def test_host_entropies_error_behaviour(engine):
    lin = np.array([0.0, 1.0, 2.0, 3.0])
    wt, inf = engine.entropies(lin, a0is0=True)
    assert np.isfinite(wt) and np.isfinite(inf)
    with pytest.raises(engine.NlcError) as e:
        engine.entropies(np.array([1.0, np.inf, 2.0]), a0is0=False)
    assert e.value.code == engine.EBLOWUP
    with pytest.raises(engine.NlcError) as e:
        engine.entropies(lin, a0is0=False, entropy_mask=np.zeros(4, dtype=np.uint8))
    assert e.value.code == engine.EINVAL and "no mode selected" in str(e.value)
    # equipartition: both entropies vanish
    wt, inf = engine.entropies(np.full(8, 0.125), a0is0=False)
    assert abs(wt) < 1e-14 and abs(inf) < 1e-14
