"""Analytic known answers on the GPU (see test_known_answers.py for the oracle's).

dDNKG with constant masses against DNKG: identical states, and equal energies in each degenerate
eigenspace.  At 256 sites the dDNKG energies come from the tensor-core projection and DNKG's from
the FFT path, so this also checks one against the other.  FPUT and Toda conserve each chain's
total momentum.
"""
import numpy as np
import pytest

from nlchains_gb300 import ic
from test_known_answers import dnkg_pair_sums, sorted_pair_sums

pytestmark = pytest.mark.gpu


def run(nlc, model, state, steps, b):
    ctx = nlc.Context(0)
    job = ctx.job(model, b)
    job.upload(state)
    job.advance(steps)
    out = job.download().reshape(state.shape)
    lin, _, _ = job.linenergies()
    job.close()
    ctx.close()
    return out, lin


@pytest.mark.parametrize("n", [16, 64, 256])
def test_ddnkg_constant_masses_is_dnkg(gpu, n):
    copies, m, steps, b = 64, 0.7, 200, 100
    state = ic.real_ensemble(n, copies, 0.3, ic.low_modes(n, kmax=3), m=m, seed=n)
    s1, e1 = run(gpu, gpu.Model("DNKG", n, copies, 0.05, m=m, beta=1.0), state, steps, b)
    s2, e2 = run(gpu, gpu.Model("dDNKG", n, copies, 0.05, masses=np.full(n, m), beta=1.0), state, steps, b)
    assert np.array_equal(s1, s2)
    p1, p2 = dnkg_pair_sums(e1), sorted_pair_sums(e2)
    assert np.abs(p1 - p2).max() <= 1e-11 * np.abs(p1).max()


@pytest.mark.parametrize("name,params", [("FPUT", dict(alpha=0.3, beta=1.0)), ("Toda", dict(alpha=0.5))])
def test_momentum_conserved(gpu, name, params):
    n, copies = 64, 32
    state = 0.3 * np.random.default_rng(5).standard_normal((copies, n, 2))
    state[:, :, 1] += 0.2
    out, _ = run(gpu, gpu.Model(name, n, copies, 0.05, **params), state, 1000, 100)
    p0, p1 = state[:, :, 1].sum(axis=1), out[:, :, 1].sum(axis=1)
    assert np.abs(p1 - p0).max() <= 1e-11 * np.abs(state[:, :, 1]).sum(axis=1).max()
