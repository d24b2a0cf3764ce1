"""Linear-mode energies and entropies on the GPU against the oracle (FP64, within 1e-10).

The reference's diagnostics (two cuFFTs + one-thread-per-mode sum for the real models, cuFFT for
DNLS, two cublasDgemm for dDNKG, then results::calc_linenergies / calc_entropies) are restated in
the oracle; the engine uses one complex FFT of phi + i pi, a Stockham shared-memory FFT and a
fixed-order on-device reduction, so agreement is to rounding, not bitwise.
"""
import numpy as np
import pytest

import oracle as O
from nlchains_gb300 import ic

pytestmark = pytest.mark.gpu

TOL = 1e-10


def diag(nlc, model, n, copies, params, state, masses=None, mask=None):
    ctx = nlc.Context(0)
    job = ctx.job(nlc.Model(model, n, copies, 0.05, masses=masses, entropy_mask=mask, **params), 10)
    job.upload(state)
    res = job.linenergies()
    res2 = job.linenergies()
    job.close()
    ctx.close()
    assert np.array_equal(res[0], res2[0]) and res[1:] == res2[1:], "diagnostics not deterministic"
    return res


def check(lin, wt, inf, exp_lin, a0is0, mask=None):
    assert np.abs(lin - exp_lin).max() <= TOL * np.abs(exp_lin).max()
    ewt, einf = O.entropies(exp_lin, a0is0, mask)
    assert abs(wt - ewt) <= TOL * max(1.0, abs(ewt))
    assert abs(inf - einf) <= TOL * max(1.0, abs(einf))


@pytest.mark.parametrize("n", [2, 3, 7, 12, 64, 86, 100, 101, 128, 509, 1021, 1024, 1536, 3583, 4096])
@pytest.mark.parametrize("model,params", [("FPUT", dict(alpha=0.0, beta=1.0)), ("DNKG", dict(m=1.0, beta=1.0)),
                                          ("Toda", dict(alpha=0.5))])
def test_real_models(gpu, model, params, n):
    copies = 37
    rng = np.random.default_rng(n)
    state = rng.standard_normal((copies, n, 2))
    lin, wt, inf = diag(gpu, model, n, copies, params, state)
    mdl = O.Model(model, n, copies, 0.05, **params)
    check(lin, wt, inf, O.linenergies(mdl, state), O.a0is0(mdl))


@pytest.mark.parametrize("n", [4, 16, 64, 100, 211, 664, 1024, 2048, 2477])
def test_dnls(gpu, n):
    copies = 29
    # a full spectrum: the WT entropy sums log e_k and is ill-conditioned for modes at rounding level
    rng = np.random.default_rng(n)
    psi = rng.standard_normal((copies, n)) + 1j * rng.standard_normal((copies, n))
    lin, wt, inf = diag(gpu, "DNLS", n, copies, dict(beta=1.0), psi.view(np.float64).reshape(copies, n, 2))
    mdl = O.Model("DNLS", n, copies, 0.05, beta=1.0)
    check(lin, wt, inf, O.linenergies(mdl, psi.view(np.float64)), True)


@pytest.mark.parametrize("n", [4, 8, 64, 256])
def test_ddnkg_projection(gpu, n):
    copies = 19
    masses = ic.masses_uniform(n, seed=n + 1)
    state = ic.ddnkg_ensemble(masses, copies, 0.5, max(2, n // 4), seed=3)
    state += 1e-3 * np.random.default_rng(n).standard_normal(state.shape)
    lin, wt, inf = diag(gpu, "dDNKG", n, copies, dict(beta=1.0), state, masses=masses)
    mdl = O.Model("dDNKG", n, copies, 0.05, beta=1.0, masses=masses)
    check(lin, wt, inf, O.linenergies(mdl, state), False)


def test_entropy_mask(gpu):
    n, copies = 64, 11
    state = np.random.default_rng(5).standard_normal((copies, n, 2))
    mask = np.zeros(n, np.uint8)
    mask[[0, 1, 2, 5, 9, 33]] = 1
    lin, wt, inf = diag(gpu, "FPUT", n, copies, dict(alpha=0.0, beta=1.0), state, mask=mask)
    mdl = O.Model("FPUT", n, copies, 0.05, alpha=0.0, beta=1.0)
    check(lin, wt, inf, O.linenergies(mdl, state), True, mask)


def test_ic_energies_land_where_requested(gpu):
    """The seeded initial ensemble of the FPUT-beta N=64 workload puts 0.1 * 64 / 8 in each mode."""
    n, copies = 64, 64
    modes = ic.low_modes(n, kmax=4, include_zero=False)
    state = ic.real_ensemble(n, copies, 0.1, modes, seed=1)
    lin, wt, inf = diag(gpu, "FPUT", n, copies, dict(alpha=0.0, beta=1.0), state)
    target = np.zeros(n)
    target[modes] = 0.1 * n / len(modes)
    assert np.abs(lin - target).max() < 1e-12


def test_blowup_is_reported(gpu):
    n, copies = 16, 4
    state = np.zeros((copies, n, 2))
    state[1, 3, 0] = np.nan
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model("FPUT", n, copies, 0.1, alpha=0.0, beta=1.0), 10)
    job.upload(state)
    with pytest.raises(gpu.NlcError) as e:
        job.linenergies()
    assert e.value.code == gpu.EBLOWUP


FP32_CASES = [("DNLS", dict(beta=1.0), 1024), ("DNLS", dict(beta=1.0), 96), ("DNLS", dict(beta=1.0), 100),
              ("DNKG", dict(m=1.0, beta=1.0), 128), ("FPUT", dict(alpha=0.0, beta=1.0), 64),
              ("Toda", dict(alpha=0.5), 1536)]


@pytest.mark.parametrize("model,params,n", FP32_CASES, ids=[f"{c[0]}-{c[2]}" for c in FP32_CASES])
def test_fp32_diagnostics_error_stated(gpu, model, params, n):
    """NLC_FLAG_FP32_DIAGNOSTICS against the FP64 oracle (radix-4, -2, -3 and -5 passes): mode
    energies within 2e-5 of the largest, the information entropy within 2e-5 relative (an FP32
    transform, the sum over chains in FP64).  The WT entropy, a sum of logs, is left out: its FP32
    error grows with the number of weak modes."""
    copies = 96
    rng = np.random.default_rng(n + 5)
    state = rng.standard_normal((copies, n, 2))
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model(model, n, copies, 0.05, flags=gpu.FLAG_FP32_DIAGNOSTICS, **params), 10)
    job.upload(state)
    lin, wt, inf = job.linenergies()
    job.close()
    ctx.close()
    mdl = O.Model(model, n, copies, 0.05, **params)
    elin = O.linenergies(mdl, state)
    _, einf = O.entropies(elin, O.a0is0(mdl))
    err = np.abs(lin - elin).max() / np.abs(elin).max()
    assert 0 < err <= 2e-5, err   # not zero: the FP32 path ran
    assert abs(inf - einf) <= 2e-5 * abs(einf)


@pytest.mark.parametrize("n", [256, 300, 1024])
def test_ddnkg_device_eigensystem_equals_host(gpu, n, monkeypatch):
    """A plan's dDNKG eigensystem solved on the GPU (cuSOLVER syevd; plans take it from 4096 sites,
    here from 256 through NLC_DEVICE_EIGEN_FROM) against the host solver (NLC_HOST_EIGEN): the same
    frequencies and, since eigenvectors are defined up to sign, the same mode energies of a state
    (both through the FP64 projection)."""
    torch = pytest.importorskip("torch")
    copies = 16
    masses = ic.masses_uniform(n, seed=n)
    state = 0.3 * np.random.default_rng(n).standard_normal((copies, n, 2))
    dev = torch.from_numpy(state).cuda()
    out = {}
    for host in (False, True):
        if host:
            monkeypatch.setenv("NLC_HOST_EIGEN", "1")
        else:
            monkeypatch.setenv("NLC_DEVICE_EIGEN_FROM", "256")
        plan = gpu.Plan(gpu.Model("dDNKG", n, copies, 0.05, masses=masses, beta=1.0, flags=gpu.FLAG_FP64_PROJECTION))
        lin = torch.zeros(n, dtype=torch.float64, device="cuda")
        plan.linenergies(dev.data_ptr(), lin.data_ptr(), 0, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        out[host] = (plan.omegas(), lin.cpu().numpy())
        plan.close()
    assert np.abs(out[False][0] - out[True][0]).max() <= 1e-12 * out[True][0].max()
    assert np.abs(out[False][1] - out[True][1]).max() <= 1e-10 * np.abs(out[True][1]).max()
