"""The C ABI library: it builds, loads, and exports every symbol include/nlchains.h declares; the
command line rejects invalid arguments before touching a GPU (CPU only)."""
import os
import re
import subprocess

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


def test_cli_usage_without_options(engine):
    r = subprocess.run([engine.EXECUTABLE_PATH, "DNLS"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "--beta" in r.stdout and "--no_linear_callback" in r.stdout
    r = subprocess.run([engine.EXECUTABLE_PATH], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "subprogram" in r.stdout
