"""Chains longer than one block holds (the reference's 16-bit --chain_length goes to 65535).

* Real models: the windowed tier.  Each block integrates a window of G E sites as a ring and keeps
  the interior the wrong ring closure cannot reach, so the result is bit-identical to the oracle's
  device operation order.  NLC_FORCE_WINDOW=<G> forces windows on short chains, so that every model
  and variant is covered at a cost the oracle can check; the natural cases run at n = 6000 .. 20000.
* DNLS and the diagnostics: transforms longer than shared memory holds run from global memory, with
  the padded convolution / Bluestein form at any length.
"""
import os

import numpy as np
import pytest

import oracle as O
from nlchains_gb300 import ic

pytestmark = pytest.mark.gpu


def run_real(nlc, name, n, copies, params, steps, b, masses=None, force_window=None, dt=0.05):
    old = os.environ.get("NLC_FORCE_WINDOW")
    if force_window:
        os.environ["NLC_FORCE_WINDOW"] = str(force_window)
    try:
        state = 0.3 * np.random.default_rng(n + copies).standard_normal((copies, n, 2))
        ctx = nlc.Context(0)
        job = ctx.job(nlc.Model(name, n, copies, dt, masses=masses, **params), b)
        job.upload(state)
        job.advance(steps)
        out = job.download().reshape(copies, n, 2)
        job.close()
        ctx.close()
    finally:
        if force_window:
            if old is None:
                del os.environ["NLC_FORCE_WINDOW"]
            else:
                os.environ["NLC_FORCE_WINDOW"] = old
    exp = O.advance(O.Model(name, n, copies, dt, masses=masses, **params), state, steps, b,
                    order=O.ORDER_DEVICE).reshape(copies, n, 2)
    return out, exp


FORCED = [
    ("FPUT", dict(alpha=0.0, beta=1.0)),
    ("FPUT", dict(alpha=0.3, beta=0.8)),
    ("DNKG", dict(m=1.0, beta=1.0)),
    ("DNKG", dict(m=0.4, beta=0.6)),
    ("Toda", dict(alpha=0.5)),
    ("Toda", dict(alpha=0.8)),
    ("dDNKG", dict(beta=1.0)),
    ("dDNKG", dict(beta=0.5)),
]


@pytest.mark.parametrize("b,steps", [(10, 30), (7, 21)])
@pytest.mark.parametrize("name,params", FORCED, ids=[f"{c[0]}-{'-'.join(f'{k}{v}' for k, v in c[1].items())}" for c in FORCED])
def test_forced_windows_bit_exact(gpu, name, params, b, steps):
    # G = 64: windows of 512 sites, 3 steps per launch (so b = 10 is 4 launches and b = 7 is 3: both
    # buffer parities), 21-site ends, 2 windows per chain of 600
    n, copies = 600, 5
    masses = ic.masses_uniform(n, seed=3) if name == "dDNKG" else None
    out, exp = run_real(gpu, name, n, copies, params, steps, b, masses=masses, force_window=64)
    assert np.array_equal(out, exp), f"{name}: windowed result differs from the oracle"


@pytest.mark.parametrize("name,n,copies,params", [
    ("DNKG", 9000, 2, dict(m=1.0, beta=1.0)),
    ("Toda", 6000, 2, dict(alpha=0.5)),
    ("FPUT", 20000, 1, dict(alpha=0.0, beta=1.0)),
    ("FPUT", 65535, 1, dict(alpha=0.2, beta=1.0)),
])
def test_long_chains_bit_exact(gpu, name, n, copies, params):
    out, exp = run_real(gpu, name, n, copies, params, 20, 10)
    assert np.array_equal(out, exp), f"{name} n={n}: differs from the oracle"


def dnls_run(nlc, n, copies, dt, beta, psi, steps, b):
    ctx = nlc.Context(0)
    job = ctx.job(nlc.Model("DNLS", n, copies, dt, beta=beta), b)
    job.upload(psi.view(np.float64).reshape(copies, n, 2))
    job.advance(steps)
    out = job.download().view(np.complex128).reshape(copies, n)
    lin, wt, inf = job.linenergies()
    job.close()
    ctx.close()
    return out, lin


@pytest.mark.parametrize("n", [8192, 9000])
def test_dnls_global_memory_transforms(gpu, n):
    copies, dt, steps, b = 2, 0.01, 4, 2
    psi = ic.dnls_ensemble(n, copies, 1.0, ic.low_modes(n, 0.1), seed=n)
    out, lin = dnls_run(gpu, n, copies, dt, 1.0, psi, steps, b)
    mdl = O.Model("DNLS", n, copies, dt, beta=1.0)
    exp = O.advance(mdl, psi.view(np.float64), steps, b).view(np.complex128).reshape(copies, n)
    assert np.abs(out - exp).max() <= 1e-12 * np.abs(exp).max()
    elin = O.linenergies(mdl, exp.view(np.float64))
    assert np.abs(lin - elin).max() <= 1e-10 * np.abs(elin).max()


@pytest.mark.parametrize("n", [7919, 10007, 65521])
def test_dnls_long_prime_linear_exact(gpu, n):
    # beta = 0: exact phase advance of every mode; prime n goes through the padded convolution of a
    # length beyond shared memory
    copies, dt, steps = 2, 0.05, 8
    rng = np.random.default_rng(n)
    psi = rng.standard_normal((copies, n)) + 1j * rng.standard_normal((copies, n))
    out, _ = dnls_run(gpu, n, copies, dt, 0.0, psi, steps, 4)
    omega = 4 * np.sin(np.pi * np.arange(n) / n) ** 2
    exp = np.fft.ifft(np.fft.fft(psi, axis=1) * np.exp(-1j * omega * dt * steps), axis=1)
    assert np.abs(out - exp).max() <= 1e-11 * np.abs(exp).max()


@pytest.mark.parametrize("n", [7919, 9000])
def test_real_diagnostics_global_memory(gpu, n):
    copies = 3
    state = np.random.default_rng(n).standard_normal((copies, n, 2))
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model("FPUT", n, copies, 0.05, alpha=0.0, beta=1.0), 10)
    job.upload(state)
    lin, wt, inf = job.linenergies()
    job.close()
    ctx.close()
    mdl = O.Model("FPUT", n, copies, 0.05, alpha=0.0, beta=1.0)
    elin = O.linenergies(mdl, state)
    assert np.abs(lin - elin).max() <= 1e-10 * np.abs(elin).max()
    ewt, einf = O.entropies(elin, O.a0is0(mdl))
    assert abs(wt - ewt) <= 1e-10 * max(1.0, abs(ewt)) and abs(inf - einf) <= 1e-10 * max(1.0, abs(einf))


@pytest.mark.parametrize("n", [700, 1800])
def test_ddnkg_projection_chunked(gpu, n):
    # the tensor-core projection over three and eight 256-site read-out chunks per sweep; the
    # expected energies come from LAPACK's eigensystem of the same operator (eigensystem.cpp:15-18)
    copies = 11
    masses = ic.masses_uniform(n, seed=n)
    state = np.random.default_rng(n).standard_normal((copies, n, 2))
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model("dDNKG", n, copies, 0.05, beta=1.0, masses=masses), 10)
    job.upload(state)
    lin, wt, inf = job.linenergies()
    job.close()
    ctx.close()
    h = np.diag(masses + 2.0)
    idx = np.arange(n)
    h[idx, (idx + 1) % n] = -1.0
    h[(idx + 1) % n, idx] = -1.0
    w, v = np.linalg.eigh(h)
    omega = np.sqrt(w)
    pphi = state[:, :, 0] @ v * omega
    ppi = state[:, :, 1] @ v
    exp = 0.5 / copies * (pphi ** 2 + ppi ** 2).sum(0)
    # two backward-stable eigensolvers agree on eigenvector k to ~ eps |H| / gap_k: closely spaced
    # eigenvalues (random masses, n = 1800) widen the bound on those modes only
    gap = np.minimum(np.abs(np.diff(w, prepend=-np.inf)), np.abs(np.diff(w, append=np.inf)))
    tol = (1e-10 + 4 * np.finfo(float).eps * np.abs(w).max() / gap) * np.abs(exp).max()
    assert (np.abs(lin - exp) <= tol).all()
    assert np.median(np.abs(lin - exp)) <= 1e-12 * np.abs(exp).max()
