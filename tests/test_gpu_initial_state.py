"""nlc_initial_state (seeded initial ensembles written on the device) against the host generator
nlchains_gb300/ic.py: the same random numbers and recipes, to rounding (a different transform)."""
import numpy as np
import pytest

import oracle as O
from nlchains_gb300 import ic

pytestmark = pytest.mark.gpu

CASES = [("DNKG", dict(m=1.0, beta=1.0), 128, 1.0), ("FPUT", dict(alpha=0.0, beta=1.0), 64, 0.0),
         ("Toda", dict(alpha=0.5), 37, 0.0), ("DNLS", dict(beta=1.0), 1024, None),
         ("DNLS", dict(beta=1.0), 211, None)]


@pytest.mark.parametrize("name,params,n,m", CASES, ids=[f"{c[0]}-{c[2]}" for c in CASES])
def test_matches_host_generator(gpu, name, params, n, m):
    """Wave numbers 0 (skipped where its frequency is 0), +-1 .. +-4 (DNLS: the lowest 10%); copies
    from an offset (first_copy); n = 37 and 211 use the padded transform."""
    torch = pytest.importorskip("torch")
    copies, seed, first, density = 33, 77, 5, 0.4
    plan = gpu.Plan(gpu.Model(name, n, copies, 0.05, **params))
    dev = torch.zeros((copies, n, 2), dtype=torch.float64, device="cuda")
    if name == "DNLS":
        modes = ic.low_modes(n, 0.1)
        exp = ic.dnls_ensemble(n, copies, density, modes, seed=seed, first_copy=first).view(np.float64)
    else:
        modes = ic.low_modes(n, kmax=4, include_zero=True)
        exp = ic.real_ensemble(n, copies, density, modes, m=m, seed=seed, first_copy=first)
    plan.initial_state(dev.data_ptr(), seed, density, modes, first_copy=first,
                       stream=torch.cuda.current_stream().cuda_stream)
    got = dev.cpu().numpy()
    plan.close()
    exp = np.asarray(exp).reshape(copies, n, 2)
    assert np.abs(got - exp).max() <= 1e-12 * np.abs(exp).max()


def test_ddnkg_mode_energies(gpu):
    """dDNKG: eigenvectors are defined up to sign, so the states of two eigensolvers may differ; the
    mode energies may not: every chain carries exactly A^2 / 2 in each excited eigenmode."""
    torch = pytest.importorskip("torch")
    n, copies, nmodes, seed, density = 64, 48, 6, 9, 0.5
    masses = ic.masses_uniform(n, seed=3)
    model = gpu.Model("dDNKG", n, copies, 0.05, masses=masses, beta=1.0)
    plan = gpu.Plan(model)
    dev = torch.zeros((copies, n, 2), dtype=torch.float64, device="cuda")
    plan.initial_state(dev.data_ptr(), seed, density, np.arange(nmodes), stream=torch.cuda.current_stream().cuda_stream)
    got = dev.cpu().numpy()
    plan.close()
    mdl = O.Model("dDNKG", n, copies, 0.05, masses=masses, beta=1.0)
    lin = O.linenergies(mdl, got)
    exp = O.linenergies(mdl, ic.ddnkg_ensemble(masses, copies, density, nmodes, seed=seed))
    assert np.abs(lin - exp).max() <= 1e-10 * np.abs(exp).max()
    assert np.abs(lin[nmodes:]).max() <= 1e-12 * np.abs(exp).max()


def test_rejects_bad_modes(gpu):
    torch = pytest.importorskip("torch")
    plan = gpu.Plan(gpu.Model("FPUT", 16, 4, 0.1, alpha=0.0, beta=1.0))
    dev = torch.zeros((4, 16, 2), dtype=torch.float64, device="cuda")
    for modes in ([16], [0]):   # out of range; only the zero-frequency mode
        with pytest.raises(gpu.NlcError) as e:
            plan.initial_state(dev.data_ptr(), 1, 0.1, modes)
        assert e.value.code == gpu.EINVAL
    plan.close()


def test_server_seeded_request_equals_job(gpu):
    """A server request submitted with a seed (its state generated on the device by the preparer)
    ends bit-identical to a job started from the same generated state, and mixes with a request
    submitted with a host state."""
    torch = pytest.importorskip("torch")
    n, copies, b, steps, seed, density = 96, 200, 10, 40, 123, 0.3
    modes = ic.low_modes(n, kmax=3, include_zero=False)
    model = gpu.Model("FPUT", n, copies, 0.05, alpha=0.2, beta=1.0)
    plan = gpu.Plan(model)
    dev = torch.zeros((copies, n, 2), dtype=torch.float64, device="cuda")
    plan.initial_state(dev.data_ptr(), seed, density, modes, stream=torch.cuda.current_stream().cuda_stream)
    init = dev.cpu().numpy()
    plan.close()
    other = 0.2 * np.random.default_rng(1).standard_normal((64, 48, 2))
    srv = gpu.Server(0)
    r1 = srv.submit_seeded(model, b, steps, seed, density, modes)
    r2 = srv.submit(gpu.Model("DNKG", 48, 64, 0.05, m=1.0, beta=1.0), b, steps, other)
    for rid in (r1, r2):
        srv.wait(rid, 60000)
    fstate, _, ents, rc = srv.result(r1)
    assert rc == gpu.OK and ents.shape == (steps // b + 1, 2)
    srv.result(r2)
    srv.close()
    ctx = gpu.Context(0)
    job = ctx.job(model, b)
    job.upload(init)
    job.advance(steps)
    assert np.array_equal(fstate.reshape(copies, n, 2), job.download().reshape(copies, n, 2))
    job.close()
    ctx.close()
