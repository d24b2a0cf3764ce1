"""The committed golden fixtures (tests/golden, written by tests/golden/make_golden.py from the oracle):
the oracle of this machine reproduces them (CPU), and the engine reproduces them (GPU): bit for bit
for the real-model integrators, to rounding for DNLS and the diagnostics."""
import glob
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "*.npz")))


def load(path):
    d = dict(np.load(path))
    d["model"] = str(d["model"])
    for k in ("n", "copies", "steps", "batching"):
        d[k] = int(d[k])
    for k in ("dt", "m", "alpha", "beta"):
        d[k] = float(d[k])
    return d


def params(d):
    p = {"DNKG": dict(m=d["m"], beta=d["beta"]), "FPUT": dict(alpha=d["alpha"], beta=d["beta"]),
         "Toda": dict(alpha=d["alpha"]), "dDNKG": dict(beta=d["beta"]), "DNLS": dict(beta=d["beta"])}
    return p[d["model"]]


def masses(d):
    return d["masses"] if d["model"] == "dDNKG" else None


def test_fixtures_present():
    assert len(GOLDEN) >= 9


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reproduces_golden(path):
    d = load(path)
    mdl = O.Model(d["model"], d["n"], d["copies"], d["dt"], masses=masses(d), **params(d))
    dev = O.advance(mdl, d["state_in"], d["steps"], d["batching"], order=O.ORDER_DEVICE).reshape(d["state_in"].shape)
    exp = d["state_device_order"]
    if d["model"] == "DNLS":
        # the oracle's DNLS uses the host C library's sincos
        assert np.abs(dev - exp).max() <= 1e-14 * np.abs(exp).max()
    else:
        # table exp, explicit operation order, no contraction: identical bits on every host
        assert np.array_equal(dev, exp)
        ref = O.advance(mdl, d["state_in"], d["steps"], d["batching"], order=O.ORDER_REFERENCE)
        assert np.abs(ref.reshape(exp.shape) - d["state_reference_order"]).max() <= 1e-14 * np.abs(exp).max()
    lin = O.linenergies(mdl, exp)
    assert np.abs(lin - d["linenergies"]).max() <= 1e-14 * np.abs(d["linenergies"]).max()
    wt, inf = O.entropies(lin, O.a0is0(mdl))
    assert np.allclose([wt, inf], d["entropies"], rtol=1e-12, atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_engine_reproduces_golden(gpu, path):
    d = load(path)
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model(d["model"], d["n"], d["copies"], d["dt"], masses=masses(d), **params(d)), d["batching"])
    job.upload(d["state_in"])
    job.advance(d["steps"])
    out = job.download().reshape(d["state_in"].shape)
    lin, wt, inf = job.linenergies()
    job.close()
    ctx.close()
    exp = d["state_device_order"]
    if d["model"] == "DNLS":
        assert np.abs(out - exp).max() <= 1e-12 * np.abs(exp).max()
    else:
        assert np.array_equal(out, exp), f"{os.path.basename(path)}: not bit-identical to the golden state"
    assert np.abs(lin - d["linenergies"]).max() <= 1e-10 * np.abs(d["linenergies"]).max()
    assert np.allclose([wt, inf], d["entropies"], rtol=1e-10, atol=1e-10)
