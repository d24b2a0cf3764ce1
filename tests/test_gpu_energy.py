"""Per-chain energies (nlc_energies / nlc_job_energies) against the oracle's restatement of the
reference post-processing's definitions (nlchains.m:40-48), and energy conservation of the
integrators: the energy drift stays at the scheme's own error level."""
import numpy as np
import pytest

import oracle as O
from nlchains_gb300 import ic

pytestmark = pytest.mark.gpu

CASES = [
    ("DNKG", dict(m=1.0, beta=1.0)),
    ("FPUT", dict(alpha=0.25, beta=0.7)),
    ("Toda", dict(alpha=0.5)),
    ("dDNKG", dict(beta=1.0)),
    ("DNLS", dict(beta=1.0)),
]


@pytest.mark.parametrize("name,params", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("n", [7, 64, 1000])
def test_energies_match_oracle(gpu, name, params, n):
    copies = 13
    masses = ic.masses_uniform(n, seed=n) if name == "dDNKG" else None
    state = 0.4 * np.random.default_rng(n).standard_normal((copies, n, 2))
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model(name, n, copies, 0.05, masses=masses, **params), 10)
    job.upload(state)
    e = job.energies()
    job.close()
    ctx.close()
    exp = O.energies(O.Model(name, n, copies, 0.05, masses=masses, **params), state)
    assert np.abs(e - exp).max() <= 1e-12 * np.abs(exp).max()


@pytest.mark.parametrize("name,params", CASES, ids=[c[0] for c in CASES])
def test_energy_drift_bounded(gpu, name, params):
    # a symplectic 6th-order integrator: the energy oscillates at O(dt^6) without secular drift
    n, copies, dt = 128, 16, 0.02
    masses = ic.masses_uniform(n, seed=1) if name == "dDNKG" else None
    if name == "DNLS":
        psi = ic.dnls_ensemble(n, copies, 1.0, ic.low_modes(n, 0.1), seed=2)
        state = np.ascontiguousarray(psi).view(np.float64).reshape(copies, n, 2)
    else:
        state = 0.3 * np.random.default_rng(3).standard_normal((copies, n, 2))
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model(name, n, copies, dt, masses=masses, **params), 100)
    job.upload(state)
    e0 = job.energies()
    job.advance(2000)
    e1 = job.energies()
    job.close()
    ctx.close()
    assert np.abs(e1 / e0 - 1).max() < 1e-8
