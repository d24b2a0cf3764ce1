"""Edge shapes of every path on the GPU: one copy, the shortest chains, lengths just past a tier or
padding boundary, against the oracle (bit-exact for the real-model integrators, to rounding
elsewhere)."""
import os

import numpy as np
import pytest

import oracle as O
from nlchains_gb300 import ic

pytestmark = pytest.mark.gpu

REAL = [("FPUT", dict(alpha=0.1, beta=1.0)), ("DNKG", dict(m=1.0, beta=1.0)), ("Toda", dict(alpha=0.5)),
        ("dDNKG", dict(beta=1.0))]


def advance_job(nlc, name, n, copies, params, state, steps, b, masses=None, flags=0):
    ctx = nlc.Context(0)
    job = ctx.job(nlc.Model(name, n, copies, 0.05, masses=masses, flags=flags, **params), b)
    job.upload(state)
    job.advance(steps)
    out = job.download().reshape(copies, n, 2)
    lin, wt, inf = job.linenergies()
    job.close()
    ctx.close()
    return out, lin


@pytest.mark.parametrize("name,params", REAL, ids=[r[0] for r in REAL])
@pytest.mark.parametrize("n,copies", [(2, 1), (3, 1), (33, 1), (129, 2), (8193, 1)])
def test_real_edges_bit_exact(gpu, name, params, n, copies):
    # 2 and 3 sites (the shortest rings), a single copy, 33 (one past a warp), 129 (one past the
    # tensor projection's 128-site threshold, a partial 64-mode tile), 8193 (one past the longest
    # single-block chain: the windowed tier)
    if name == "dDNKG" and n > 1000:
        pytest.skip("the host eigensystem of 8193 sites takes minutes")
    masses = ic.masses_uniform(n, seed=n) if name == "dDNKG" else None
    state = 0.3 * np.random.default_rng(n + copies).standard_normal((copies, n, 2))
    out, lin = advance_job(gpu, name, n, copies, params, state, 20, 10, masses)
    mdl = O.Model(name, n, copies, 0.05, masses=masses, **params)
    exp = O.advance(mdl, state, 20, 10, order=O.ORDER_DEVICE).reshape(copies, n, 2)
    assert np.array_equal(out, exp)
    elin = O.linenergies(mdl, exp)
    assert np.abs(lin - elin).max() <= 1e-10 * np.abs(elin).max()


@pytest.mark.parametrize("n,copies", [(2, 1), (5, 1), (257, 1), (7201, 1)])
def test_dnls_edges(gpu, n, copies):
    # 2 and 5 sites, a single copy, 257 (one past the warp-team pass length, prime: padded
    # convolution), 7201 (one past the shared-memory pass length: global-memory passes)
    rng = np.random.default_rng(n)
    psi = rng.standard_normal((copies, n)) + 1j * rng.standard_normal((copies, n))
    state = np.ascontiguousarray(psi).view(np.float64).reshape(copies, n, 2)
    steps, b = (4, 2) if n > 1000 else (20, 10)
    out, lin = advance_job(gpu, "DNLS", n, copies, dict(beta=1.0), state, steps, b)
    mdl = O.Model("DNLS", n, copies, 0.05, beta=1.0)
    exp = O.advance(mdl, state.reshape(copies, n * 2), steps, b).reshape(copies, n, 2)
    assert np.abs(out - exp).max() <= 1e-12 * np.abs(exp).max()
    elin = O.linenergies(mdl, exp)
    assert np.abs(lin - elin).max() <= 1e-10 * np.abs(elin).max()


def test_server_single_copy_requests(gpu):
    # one-copy requests of every model in one server: each equals its run alone
    srv = gpu.Server(0)
    reqs = []
    for i, (name, params) in enumerate(REAL + [("DNLS", dict(beta=1.0))]):
        n = 40 + i
        masses = ic.masses_uniform(n, seed=i) if name == "dDNKG" else None
        state = 0.3 * np.random.default_rng(i).standard_normal((1, n, 2))
        model = gpu.Model(name, n, 1, 0.05, masses=masses, **params)
        reqs.append((srv.submit(model, 5, 20, state), name, n, params, masses, state))
    for rid, name, n, params, masses, state in reqs:
        srv.wait(rid, 60000)
        fstate, _, ents, rc = srv.result(rid)
        assert rc == gpu.OK and ents.shape == (5, 2)
        out, _ = advance_job(gpu, name, n, 1, params, state, 20, 5, masses)
        assert np.array_equal(fstate.reshape(1, n, 2), out)
    srv.close()


def test_rejects_invalid_models(gpu):
    ctx = gpu.Context(0)
    for bad in (gpu.Model("FPUT", 1, 4, 0.1, beta=1.0), gpu.Model("FPUT", 16, 0, 0.1, beta=1.0),
                gpu.Model("Toda", 16, 4, 0.1, alpha=0.0)):
        with pytest.raises(gpu.NlcError) as e:
            ctx.job(bad, 10)
        assert e.value.code == gpu.EINVAL
    ctx.close()
