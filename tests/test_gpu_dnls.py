"""DNLS split-step integrator on the GPU against the oracle and against exact known answers."""
import numpy as np
import pytest

import oracle as O
from nlchains_gb300 import ic

pytestmark = pytest.mark.gpu


# the linear sub-steps as real-space stencils (the default where dt and n allow) and through transforms
FORMS = {"stencil": 0, "fourier": 512}


def run(nlc, n, copies, dt, beta, psi, steps, batching, flags=0):
    ctx = nlc.Context(0)
    job = ctx.job(nlc.Model("DNLS", n, copies, dt, beta=beta, flags=flags), batching)
    job.upload(psi.view(np.float64).reshape(copies, n, 2))
    job.advance(steps)
    out = job.download().view(np.complex128).reshape(copies, n)
    job.close()
    ctx.close()
    return out


# 70 = 2 x 5 x 7 (direct radix-5 and radix-7 passes), 39 / 86 (factors 13, 43) and 97 / 211 / 997 /
# 3001 prime (Bluestein), 1000 smooth: every FFT path and every team width of the shared-memory step
# 664 pads to 1536 points: exactly 48 KiB of dynamic shared memory per block, plus the static part
# the stencil form: 16 (one lane of 16 sites), 39 / 53 .. 211 / 256 / 512 (5 .. 32 lanes of a warp, 8,
# 12 or 16 sites), 664 .. 3001 (a block of 56 .. 188 lanes); 2, 8, 12 are too short for its radius
# and take the Fourier form either way
@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("n", [2, 8, 12, 16, 39, 64, 70, 86, 97, 100, 211, 256, 512, 664, 997, 1000, 1024, 2048,
                               3001])
def test_against_oracle(gpu, n, form):
    copies, dt = 11, 0.01
    steps, b = (20, 10) if n <= 2048 else (4, 2)   # the oracle's prime-length DFT is O(n^2)
    if n > 2048:
        copies = 3
    psi = ic.dnls_ensemble(n, copies, 1.0, ic.low_modes(n, 0.1), seed=n)
    tier = gpu.Plan(gpu.Model("DNLS", n, copies, dt, beta=1.0, flags=FORMS[form])).shape()["tier"]
    assert tier == (5 if form == "stencil" and n >= 16 else 3)
    out = run(gpu, n, copies, dt, 1.0, psi, steps, b, FORMS[form])
    mdl = O.Model("DNLS", n, copies, dt, beta=1.0)
    exp = O.advance(mdl, psi.view(np.float64), steps, b).view(np.complex128).reshape(copies, n)
    # different FFT algorithms and sincos implementations: agreement to rounding
    assert np.abs(out - exp).max() <= 1e-12 * np.abs(exp).max()


# Fourier form: 128 direct passes; 97, 211, 1021 (prime) padded cyclic convolutions.  Stencil form
# (radius 11 at dt = 0.05): 128, 211 and 1021 on lanes of 16 sites; 97 has no shape at that radius
# and keeps the Fourier form
@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("n", [128, 97, 211, 1021])
def test_linear_exact_phase_advance(gpu, n, form):
    copies, dt, steps = 5, 0.05, 40
    rng = np.random.default_rng(1)
    psi = rng.standard_normal((copies, n)) + 1j * rng.standard_normal((copies, n))
    out = run(gpu, n, copies, dt, 0.0, psi, steps, 20, FORMS[form])
    omega = 4 * np.sin(np.pi * np.arange(n) / n) ** 2
    exp = np.fft.ifft(np.fft.fft(psi, axis=1) * np.exp(-1j * omega * dt * steps), axis=1)
    assert np.abs(out - exp).max() <= 1e-12 * np.abs(exp).max()


@pytest.mark.parametrize("form", FORMS)
def test_norm_and_energy_conservation(gpu, form):
    n, copies = 1024, 8
    psi = ic.dnls_ensemble(n, copies, 1.0, ic.low_modes(n, 0.1), seed=7)
    out = run(gpu, n, copies, 0.01, 1.0, psi, 200, 100, FORMS[form])
    assert np.allclose((np.abs(out) ** 2).sum(1), (np.abs(psi) ** 2).sum(1), rtol=1e-12)
    mdl = O.Model("DNLS", n, copies, 0.01, beta=1.0)
    e0 = O.energies(mdl, psi.view(np.float64))
    e1 = O.energies(mdl, out.view(np.float64))
    assert np.abs(e1 / e0 - 1).max() < 1e-8


def test_elementwise_operators(gpu):
    torch = pytest.importorskip("torch")
    n, copies = 32, 3
    rng = np.random.default_rng(2)
    psi = rng.standard_normal((copies, n)) + 1j * rng.standard_normal((copies, n))
    plan = gpu.Plan(gpu.Model("DNLS", n, copies, 0.01, beta=1.0))
    dev = torch.from_numpy(psi.copy()).cuda()
    plan.dnls_evolve_nonlinear(dev.data_ptr(), 0.37, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    exp = psi * np.exp(-1j * 0.37 * np.abs(psi) ** 2)
    assert np.abs(dev.cpu().numpy() - exp).max() < 1e-14 * np.abs(exp).max()
    table = np.exp(-1j * rng.random(n))
    tdev = torch.from_numpy(table).cuda()
    plan.dnls_evolve_linear(dev.data_ptr(), tdev.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.abs(dev.cpu().numpy() - exp * table[None, :]).max() < 1e-14 * np.abs(exp).max()


def test_phase_rotation_accuracy(gpu):
    """The sincos of the phase rotation against numpy for |theta| from 1e-8 to 1e7 (a Taylor series
    below 2^-4, the table method above, the library sincos from 2^20; coef 0.0156 and 0.03 put warps
    on both sides of 2^-4): psi = (x, 0) with x a 13-bit dyadic number in [0.5, 2], so |psi|^2 is
    exact, theta = -coef x^2 is rounded once on both sides, and the result must be
    x (cos theta, sin theta) to a few ulp."""
    torch = pytest.importorskip("torch")
    n, copies = 64, 64
    x = np.round(np.random.default_rng(4).uniform(0.5, 2.0, n * copies) * 2 ** 12) / 2 ** 12
    plan = gpu.Plan(gpu.Model("DNLS", n, copies, 0.01, beta=1.0))
    for coef in (1e-8, 1e-3, 0.0156, 0.03, 0.37, 3.0, 123.0, 4.1e4, 3e6):
        dev = torch.from_numpy(np.stack([x, np.zeros_like(x)], axis=1).copy()).cuda()
        plan.dnls_evolve_nonlinear(dev.data_ptr(), coef, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        out = dev.cpu().numpy()
        theta = -coef * (x * x)
        err = max(np.abs(out[:, 0] - x * np.cos(theta)).max(), np.abs(out[:, 1] - x * np.sin(theta)).max())
        assert err <= 4 * 2.0 ** -52, (coef, err)


def test_long_run_conservation(gpu):
    """10^4 steps of the DNLS benchmark configuration (N = 1024, beta = 1, dt = 0.01, norm density 1
    over the lowest 10% of modes) on 32 copies: the norm of every chain, exact in exact arithmetic
    (the phase rotation and the unitary propagator both keep it), holds to rounding, and the
    energy drift stays bounded."""
    n, copies, steps = 1024, 32, 10000
    psi = ic.dnls_ensemble(n, copies, 1.0, ic.low_modes(n, 0.1), seed=9)
    out = run(gpu, n, copies, 0.01, 1.0, psi, steps, 100)
    norm0, norm1 = (np.abs(psi) ** 2).sum(1), (np.abs(out) ** 2).sum(1)
    assert np.abs(norm1 / norm0 - 1).max() < 1e-11
    mdl = O.Model("DNLS", n, copies, 0.01, beta=1.0)
    e0 = O.energies(mdl, psi.view(np.float64))
    e1 = O.energies(mdl, out.view(np.float64))
    assert np.abs(e1 / e0 - 1).max() < 1e-7


@pytest.mark.parametrize("n", [53, 1024, 2953])
def test_stencil_and_fourier_forms_agree(gpu, n):
    """The same split step with the linear sub-steps as stencils and through transforms (for the
    prime lengths, padded convolutions): agreement to rounding after 50 steps of the DNLS
    benchmark's dynamics, in one launch and in launches of 10 steps (merged rotations between them)."""
    copies, dt = 6, 0.01
    psi = ic.dnls_ensemble(n, copies, 1.0, ic.low_modes(n, 0.1), seed=n + 1)
    a = run(gpu, n, copies, dt, 1.0, psi, 50, 50)
    b = run(gpu, n, copies, dt, 1.0, psi, 50, 10)
    f = run(gpu, n, copies, dt, 1.0, psi, 50, 10, FORMS["fourier"])
    assert np.abs(a - f).max() <= 1e-12 * np.abs(f).max()
    assert np.abs(a - b).max() <= 1e-13 * np.abs(f).max()


def test_form_selection(gpu):
    """The stencil form where its radius (dt) and the chain length allow, the Fourier form otherwise
    or on request."""
    def tier(n, dt, flags=0):
        return gpu.Plan(gpu.Model("DNLS", n, 4, dt, beta=1.0, flags=flags)).shape()["tier"]
    assert tier(1024, 0.01) == 5 and tier(2953, 0.01) == 5 and tier(53, 0.01) == 5
    assert tier(1024, 0.01, FORMS["fourier"]) == 3
    assert tier(1024, 0.2) == 3                 # taps beyond radius 11 above 2^-64
    assert tier(12, 0.01) == 3                  # shorter than 2R + 2
    assert tier(8192, 0.01) == 6                # beyond 256 lanes of 16 sites: windows
    assert tier(8192, 0.2) == 3
    shape = gpu.Plan(gpu.Model("DNLS", 2953, 4, 0.01, beta=1.0)).shape()
    assert shape["sites_per_lane"] == 16 and shape["lanes_per_chain"] == 185 and shape["threads"] == 192
    # windows: the width with the least work per chain (windows x window length)
    for n, lanes in ((8192, 192), (16384, 224), (65535, 96)):
        shape = gpu.Plan(gpu.Model("DNLS", n, 4, 0.01, beta=1.0)).shape()
        assert shape["tier"] == 6 and shape["lanes_per_chain"] == lanes and shape["sites_per_lane"] == 16, (n, shape)


# (n, dt, sites per lane) -> every instantiation: radius 7 (dt = 0.01) with 8, 12, 16 sites and
# radius 11 (dt = 0.05) with 12, 16, each on lanes of one warp (team) and on a block
INSTANTIATIONS = [(62, 0.01, 8, "team"), (512, 0.01, 8, "block"), (128, 0.01, 12, "team"),
                  (1024, 0.01, 12, "block"), (256, 0.01, 16, "team"), (1024, 0.01, 16, "block"),
                  (128, 0.05, 12, "team"), (1000, 0.05, 12, "block"), (128, 0.05, 16, "team"),
                  (1021, 0.05, 16, "block")]


@pytest.mark.parametrize("n,dt,sites,kind", INSTANTIATIONS)
def test_every_stencil_instantiation(gpu, monkeypatch, n, dt, sites, kind):
    monkeypatch.setenv("NLC_DNLS_SITES", str(sites))
    copies = 9
    shape = gpu.Plan(gpu.Model("DNLS", n, copies, dt, beta=1.0)).shape()
    assert shape["tier"] == 5 and shape["sites_per_lane"] == sites
    assert (shape["lanes_per_chain"] <= 32) == (kind == "team")
    psi = ic.dnls_ensemble(n, copies, 1.0, ic.low_modes(n, 0.1), seed=sites + n)
    a = run(gpu, n, copies, dt, 1.0, psi, 20, 10)
    f = run(gpu, n, copies, dt, 1.0, psi, 20, 10, FORMS["fourier"])
    assert np.abs(a - f).max() <= 1e-12 * np.abs(f).max()


@pytest.mark.parametrize("n,sites", [(16, 0), (53, 0), (62, 8), (62, 16), (128, 12), (1024, 8), (1024, 12),
                                     (1024, 16), (2953, 0)])
def test_stencil_form_bit_exact_against_the_oracle(gpu, monkeypatch, n, sites):
    """The stencil form against the oracle's replay of it (NLO_ORDER_STENCIL): bit for bit, whatever
    the launch shape (lanes of a warp or a block, 8, 12 or 16 sites per lane), across launches."""
    if sites:
        monkeypatch.setenv("NLC_DNLS_SITES", str(sites))
    copies, dt, steps, b = (5, 0.01, 20, 10) if n < 2000 else (2, 0.01, 4, 2)
    assert gpu.Plan(gpu.Model("DNLS", n, copies, dt, beta=1.0)).shape()["tier"] == 5
    psi = ic.dnls_ensemble(n, copies, 1.0, ic.low_modes(n, 0.1), seed=3 * n + sites)
    out = run(gpu, n, copies, dt, 1.0, psi, steps, b)
    exp = O.advance(O.Model("DNLS", n, copies, dt, beta=1.0), np.ascontiguousarray(psi).view(np.float64), steps, b,
                    order=O.ORDER_STENCIL).view(np.complex128).reshape(copies, n)
    assert np.array_equal(out, exp), np.abs(out - exp).max()


@pytest.mark.parametrize("n,dt,force,copies,steps,b", [
    (5000, 0.01, None, 3, 20, 10),     # windows of 192 lanes x 16 sites, 3 steps per launch (3 + 3 + 3 + 1)
    (5000, 0.05, None, 2, 6, 3),       # radius 11: 1 step per launch
    (1500, 0.01, "64", 4, 9, 3),       # forced windows of 64 lanes on a shorter chain, 1 step per launch
    (65535, 0.01, None, 1, 4, 4),      # the longest 16-bit chain
])
def test_windowed_stencil_bit_exact(gpu, monkeypatch, n, dt, force, copies, steps, b):
    """Chains beyond one block in overlapping windows (tier 6): bit for bit the oracle's replay of the
    stencil form, over launches that leave the batch open and continue it."""
    if force:
        monkeypatch.setenv("NLC_FORCE_WINDOW", force)
    assert gpu.Plan(gpu.Model("DNLS", n, copies, dt, beta=1.0)).shape()["tier"] == 6
    psi = ic.dnls_ensemble(n, copies, 1.0, ic.low_modes(n, 0.1), seed=n + 7)
    out = run(gpu, n, copies, dt, 1.0, psi, steps, b)
    exp = O.advance(O.Model("DNLS", n, copies, dt, beta=1.0), np.ascontiguousarray(psi).view(np.float64), steps, b,
                    order=O.ORDER_STENCIL).view(np.complex128).reshape(copies, n)
    assert np.array_equal(out, exp), np.abs(out - exp).max()
