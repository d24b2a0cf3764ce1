"""dDNKG mode projection on the tensor cores (tcgen05, 7-slice BF16 split with FP32 accumulation
and FP64 recombination; the default from 128 sites) against the FP64 CUDA-core projection and a
LAPACK-based reference."""
import numpy as np
import pytest

from nlchains_gb300 import ic

pytestmark = pytest.mark.gpu


def lin_of(nlc, n, copies, state, masses, flags):
    ctx = nlc.Context(0)
    job = ctx.job(nlc.Model("dDNKG", n, copies, 0.05, beta=1.0, masses=masses, flags=flags), 10)
    job.upload(state)
    lin, wt, inf = job.linenergies()
    lin2, wt2, inf2 = job.linenergies()
    job.close()
    ctx.close()
    assert np.array_equal(lin, lin2) and wt == wt2, "not deterministic"
    return lin, wt, inf


# 16 sites: one 16-site stage, fewer stages than the pipeline holds; 300 and 700 sites: K in two
# and three read-out chunks; 1100: five chunks, the last one 6 stages; 4096 copies: 64 row tiles
@pytest.mark.parametrize("n,copies", [(16, 19), (100, 64), (256, 4096), (300, 33), (700, 11), (1100, 70)])
def test_tensor_projection_matches_fp64(gpu, n, copies):
    masses = ic.masses_uniform(n, seed=n)
    state = np.random.default_rng(n + copies).standard_normal((copies, n, 2))
    l64, w64, i64 = lin_of(gpu, n, copies, state, masses, gpu.FLAG_FP64_PROJECTION)
    ltc, wtc, itc = lin_of(gpu, n, copies, state, masses, gpu.FLAG_TENSOR_PROJECTION)
    assert np.abs(ltc - l64).max() <= 1e-13 * np.abs(l64).max()
    assert abs(wtc - w64) <= 1e-12 * max(1.0, abs(w64)) and abs(itc - i64) <= 1e-12 * max(1.0, abs(i64))


def test_tensor_projection_against_lapack(gpu):
    n, copies = 256, 512
    masses = ic.masses_uniform(n, seed=7)
    state = np.random.default_rng(8).standard_normal((copies, n, 2))
    lin, _, _ = lin_of(gpu, n, copies, state, masses, gpu.FLAG_TENSOR_PROJECTION)
    h = np.diag(masses + 2.0)
    idx = np.arange(n)
    h[idx, (idx + 1) % n] = -1.0
    h[(idx + 1) % n, idx] = -1.0
    w, v = np.linalg.eigh(h)
    exp = 0.5 / copies * ((state[:, :, 0] @ v * np.sqrt(w)) ** 2 + (state[:, :, 1] @ v) ** 2).sum(0)
    # eigenvectors of two backward-stable solvers agree to ~ eps |H| / gap on closely spaced modes
    gap = np.minimum(np.abs(np.diff(w, prepend=-np.inf)), np.abs(np.diff(w, append=np.inf)))
    tol = (1e-11 + 4 * np.finfo(float).eps * np.abs(w).max() / gap) * np.abs(exp).max()
    assert (np.abs(lin - exp) <= tol).all()


def test_tensor_projection_wide_dynamic_range(gpu):
    # chains whose amplitudes span twelve orders of magnitude, and an all-zero chain: the per-row
    # power-of-two scaling keeps the small ones, the zero chain contributes nothing
    n, copies = 64, 40
    masses = ic.masses_uniform(n, seed=9)
    rng = np.random.default_rng(10)
    state = rng.standard_normal((copies, n, 2)) * 10.0 ** rng.uniform(-6, 6, (copies, 1, 1))
    state[3] = 0.0
    l64, _, _ = lin_of(gpu, n, copies, state, masses, gpu.FLAG_FP64_PROJECTION)
    ltc, _, _ = lin_of(gpu, n, copies, state, masses, gpu.FLAG_TENSOR_PROJECTION)
    assert np.abs(ltc - l64).max() <= 1e-13 * np.abs(l64).max()


@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_tensor_projection_reports_blowup(gpu, bad):
    # a non-finite site (a blown-up chain) must surface as NLC_EBLOWUP, the reference's quit condition
    n, copies = 256, 16
    masses = ic.masses_uniform(n, seed=11)
    state = np.random.default_rng(12).standard_normal((copies, n, 2))
    state[5, 17, 1] = bad
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model("dDNKG", n, copies, 0.05, beta=1.0, masses=masses, flags=gpu.FLAG_TENSOR_PROJECTION), 10)
    job.upload(state)
    with pytest.raises(gpu.NlcError) as e:
        job.linenergies()
    assert e.value.code == gpu.EBLOWUP
    job.close()
    ctx.close()


@pytest.mark.parametrize("n,copies", [(256, 512), (300, 33)])
def test_bf16x3_projection_error_stated(gpu, n, copies):
    # 3 BF16 slices (6 tensor products) instead of 7: mode energies within 1e-6 of the FP64 ones
    # (the split keeps ~24 bits of every value), entropies within 1e-6
    masses = ic.masses_uniform(n, seed=n)
    state = np.random.default_rng(n).standard_normal((copies, n, 2))
    l64, w64, i64 = lin_of(gpu, n, copies, state, masses, gpu.FLAG_FP64_PROJECTION)
    l3, w3, i3 = lin_of(gpu, n, copies, state, masses, gpu.FLAG_BF16X3_PROJECTION)
    err = np.abs(l3 - l64).max() / np.abs(l64).max()
    assert 0 < err <= 1e-6
    assert abs(w3 - w64) <= 1e-6 * max(1.0, abs(w64)) and abs(i3 - i64) <= 1e-6 * max(1.0, abs(i64))


# 256 and 700 sites: one and three read-out chunks per sweep
@pytest.mark.parametrize("n,copies", [(256, 64), (700, 16)])
def test_projection_wait_timeout_reported(gpu, monkeypatch, n, copies):
    """A projection whose bounded wait runs out (tests only: each block first waits 1 ms on a barrier
    nothing arrives at) reports NLC_ETIMEDOUT, not a blow-up, and leaves the context usable: a plan
    made afterwards without the test wait gives the normal result."""
    masses = ic.masses_uniform(n, seed=9)
    state = ic.ddnkg_ensemble(masses, copies, 0.5, 8, seed=9)
    model = gpu.Model("dDNKG", n, copies, 0.05, masses=masses, beta=1.0)
    ctx = gpu.Context(0)
    monkeypatch.setenv("NLC_TEST_TC_WAIT", "1")
    bad = ctx.job(model, 10)
    monkeypatch.delenv("NLC_TEST_TC_WAIT")
    bad.upload(state)
    for _ in range(2):
        with pytest.raises(gpu.NlcError) as e:
            bad.linenergies()
        assert e.value.code == gpu.ETIMEDOUT
    good = ctx.job(model, 10)
    good.upload(state)
    lin, wt, inf = good.linenergies()
    assert np.all(np.isfinite(lin)) and np.isfinite(wt) and np.isfinite(inf)
    bad.close()
    good.close()
    ctx.close()
