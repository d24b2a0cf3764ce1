"""The engine against the reference itself, on the GPU.

1. The reference's own GPU kernels (its move<model>, make_linenergies and DNLS kernels, compiled
   unmodified from its sources into oracle/_ref/ref_gpu_n<N>.fatbin, launched by
   oracle/ref_shim/ref_gpu_host.cpp with cuFFT and cuBLAS as the reference calls them), on identical
   seeded ensembles at the benchmark configurations' shapes and parameters: the state after 10^3
   steps agrees to 1e-12 (max-norm, relative to the largest coordinate), the mode energies and
   entropies of each side's result to 1e-10.
2. The reference's CPU program (tests/golden/reference): every sample's mode energies and entropies
   to 1e-10, the real-model states after 10^3 steps to 1e-12.
3. DNLS, whose dynamics at the N = 1024 configuration amplifies any rounding difference by about
   10^3 over 10^3 steps (the reference's own CPU and GPU paths end 2e-9 apart): to 1e-12 of the
   reference's GPU kernels after 10^2 steps, and, against an extended-precision run of the same
   split step (tests/golden/extended), at least as accurate as the reference's GPU kernels at every
   checkpoint up to 10^3 steps, its energy drift as close to the extended run's as theirs.
4. Long runs: the dDNKG configuration over its full 5 10^4 steps, bit-identical to the oracle's
   device order and to the reference's own warp kernel at every sample, mode energies and entropies
   within 1e-10, drift as the reference's CPU arithmetic; DNLS over 10^4 steps (every mode excited),
   where trajectories of any two implementations part within 4 10^3 steps, with an energy drift no
   larger than the reference kernels'.
"""
import glob
import os

import numpy as np
import pytest

import oracle as O
from nlchains_gb300 import ic

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
STATE_TOL = 1e-12   # relative max-norm state agreement after 10^3 steps
DIAG_TOL = 1e-10    # mode energies (relative to the largest) and entropies


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def refgpu(n_opt):
    if not O.RefGPU.available(n_opt):
        pytest.skip(f"oracle/_ref/ref_gpu_n{n_opt}.fatbin was not built from the reference's sources")
    return O.RefGPU(n_opt)


def seeded_state(model, n, copies, recipe, params, masses=None, seed=12345):
    if model == "dDNKG":
        return ic.ddnkg_ensemble(masses, copies, recipe["eps"], recipe["nmodes"], seed=seed)
    modes = ic.low_modes(n, recipe.get("fraction"), kmax=recipe.get("kmax"), include_zero=recipe["include_zero"])
    if model == "DNLS":
        psi = ic.dnls_ensemble(n, copies, recipe["eps"], modes, seed=seed)
        return np.ascontiguousarray(psi).view(np.float64).reshape(copies, n, 2)
    return ic.real_ensemble(n, copies, recipe["eps"], modes, m=params.get("m", 0.0), seed=seed)


def engine_run(gpu, model, n, copies, dt, params, masses, state, steps, batching, sample_every=None):
    """The engine through the job API: final state, final (lin, WT, INF) and the samples on the way."""
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model(model, n, copies, dt, masses=masses, **params), batching)
    job.upload(state)
    samples = []
    if sample_every:
        for t in range(0, steps + 1, sample_every):
            samples.append(job.linenergies())
            if t < steps:
                job.advance(sample_every)
    else:
        job.advance(steps)
    out = job.download().reshape(state.shape)
    lin = job.linenergies()
    job.close()
    ctx.close()
    return out, lin, samples


def reference_run(torch, ref, mdl, state, steps, batching):
    dev = torch.from_numpy(np.ascontiguousarray(state).copy()).cuda()
    if mdl.model == O.DNLS:
        ref.dnls_advance(mdl, dev.data_ptr(), steps, batching)
    else:
        ref.advance(mdl, dev.data_ptr(), steps, batching)
    lin = ref.linenergies(mdl, dev.data_ptr())
    return dev.cpu().numpy().reshape(state.shape), lin


def well_conditioned(lin):
    return lin[1:].min() > 1e-8 * lin.max()


def check_diagnostics(lin, wt, inf, ref_lin, a0is0, what):
    ref_wt, ref_inf = O.entropies(ref_lin, a0is0)
    assert rel(lin, ref_lin) <= DIAG_TOL, f"{what}: mode energies differ by {rel(lin, ref_lin):.2e}"
    assert abs(inf - ref_inf) <= DIAG_TOL * max(1.0, abs(ref_inf)), f"{what}: information entropy"
    if well_conditioned(ref_lin):
        assert abs(wt - ref_wt) <= DIAG_TOL * max(1.0, abs(ref_wt)), f"{what}: WT entropy"


# (id, model, n, copies, dt, params, optimised length of the reference build, initial-state recipe):
# the benchmark configurations' shapes and parameters (all their copies where it is cheap), plus
# the reference's thread-per-chain (n < 32) and split (n other than the optimised length) tiers
REAL_CASES = [
    ("FPUT-n64-config", "FPUT", 64, 1024, 0.1, dict(alpha=0.0, beta=1.0), 64,
     dict(eps=0.1, kmax=4, include_zero=False)),
    ("DNKG-n128-config", "DNKG", 128, 4096, 0.05, dict(m=1.0, beta=1.0), 128,
     dict(eps=0.5, fraction=0.08, include_zero=True)),
    ("Toda-n128-config", "Toda", 128, 4096, 0.05, dict(alpha=0.5), 128,
     dict(eps=0.5, fraction=0.08, include_zero=False)),
    ("dDNKG-n256-config", "dDNKG", 256, 4096, 0.05, dict(beta=1.0), 256, dict(eps=0.5, nmodes=20)),
    ("FPUT-n37-split", "FPUT", 37, 256, 0.1, dict(alpha=0.25, beta=1.0), 64, dict(eps=0.1, kmax=3, include_zero=False)),
    ("Toda-n100-split", "Toda", 100, 256, 0.05, dict(alpha=0.5), 128, dict(eps=0.5, kmax=4, include_zero=False)),
    ("DNKG-n12-thread", "DNKG", 12, 512, 0.05, dict(m=0.5, beta=1.0), 64, dict(eps=0.5, kmax=5, include_zero=True)),
    ("FPUT-n5-thread", "FPUT", 5, 512, 0.1, dict(alpha=0.25, beta=1.0), 64, dict(eps=0.1, kmax=2, include_zero=False)),
    ("dDNKG-n20-thread", "dDNKG", 20, 256, 0.05, dict(beta=1.0), 256, dict(eps=0.5, nmodes=4)),
    ("dDNKG-n40-split", "dDNKG", 40, 256, 0.05, dict(beta=1.0), 256, dict(eps=0.5, nmodes=4)),
]


@pytest.mark.parametrize("case", REAL_CASES, ids=lambda c: c[0])
def test_engine_matches_reference_gpu_kernels_after_1000_steps(gpu, case):
    torch = pytest.importorskip("torch")
    _, model, n, copies, dt, params, n_opt, recipe = case
    ref = refgpu(n_opt)
    masses = ic.masses_uniform(n, seed=777) if model == "dDNKG" else None
    state = seeded_state(model, n, copies, recipe, params, masses)
    mdl = O.Model(model, n, copies, dt, masses=masses, **params)
    # identical input: diagnostics of the two implementations on the same bytes
    dev = torch.from_numpy(state.copy()).cuda()
    lin0_ref = ref.linenergies(mdl, dev.data_ptr())
    _, _, first = engine_run(gpu, model, n, copies, dt, params, masses, state, 0, 100, sample_every=100)
    assert rel(first[0][0], lin0_ref) <= 1e-12
    out, (lin, wt, inf), _ = engine_run(gpu, model, n, copies, dt, params, masses, state, 1000, 100)
    ref_out, ref_lin = reference_run(torch, ref, mdl, state, 1000, 100)
    ref.close()
    d = rel(out, ref_out)
    print(f"{case[0]}: engine vs reference kernels after 10^3 steps {d:.2e}")
    assert d <= STATE_TOL
    check_diagnostics(lin, wt, inf, ref_lin, O.a0is0(mdl), case[0])


REFERENCE_FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "reference", "*.npz")))


def load(path):
    d = dict(np.load(path))
    for k in ("name", "model"):
        d[k] = str(d[k])
    for k in ("n", "copies", "steps", "batching"):
        d[k] = int(d[k])
    for k in ("dt", "m", "alpha", "beta"):
        d[k] = float(d[k])
    d["params"] = {"DNKG": dict(m=d["m"], beta=d["beta"]), "FPUT": dict(alpha=d["alpha"], beta=d["beta"]),
                   "Toda": dict(alpha=d["alpha"]), "dDNKG": dict(beta=d["beta"]),
                   "DNLS": dict(beta=d["beta"])}[d["model"]]
    return d


@pytest.mark.parametrize("path", REFERENCE_FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_engine_matches_reference_cpu_program(gpu, path):
    d = load(path)
    masses = d["masses"] if d["model"] == "dDNKG" else None
    out, _, samples = engine_run(gpu, d["model"], d["n"], d["copies"], d["dt"], d["params"], masses, d["state_in"],
                                 d["steps"], d["batching"], sample_every=d["batching"])
    mdl = O.Model(d["model"], d["n"], d["copies"], d["dt"], masses=masses, **d["params"])
    dnls = d["model"] == "DNLS"
    for s, (lin, wt, inf) in enumerate(samples):
        t = s * d["batching"]
        if dnls and t > 100:
            break   # past 10^2 steps the reference CPU's rotation shortcut and chaos dominate (see module doc)
        assert d["entropy"][s][0] == t * d["dt"]
        check_diagnostics(lin, wt, inf, d["linenergies"][s], O.a0is0(mdl), f"{d['name']} t={t}")
    if not dnls:
        assert rel(out, d["state_out"]) <= STATE_TOL


EXTENDED = sorted(glob.glob(os.path.join(HERE, "golden", "extended", "*.npz")))


# the linear sub-steps as real-space stencils (the default) and through transforms
DNLS_FORMS = {"stencil": 0, "fourier": 512}


@pytest.mark.parametrize("form", DNLS_FORMS)
@pytest.mark.parametrize("path", EXTENDED, ids=lambda p: os.path.basename(p)[:-4])
def test_dnls_as_accurate_as_reference_kernels(gpu, path, form):
    torch = pytest.importorskip("torch")
    d = dict(np.load(path))
    n, copies, dt, beta, b = int(d["n"]), int(d["copies"]), float(d["dt"]), float(d["beta"]), int(d["batching"])
    ref = refgpu(64)
    mdl = O.Model("DNLS", n, copies, dt, beta=beta)
    state = d["state_in"]
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model("DNLS", n, copies, dt, beta=beta, flags=DNLS_FORMS[form]), b)
    job.upload(state)
    dev = torch.from_numpy(state.copy()).cuda()
    e0 = O.energies(mdl, state)
    t = 0
    for cp in d["checkpoints"]:
        cp = int(cp)
        job.advance(cp - t)
        ref.dnls_advance(mdl, dev.data_ptr(), cp - t, b)
        t = cp
        eng, rgpu, ext = job.download().reshape(state.shape), dev.cpu().numpy().reshape(state.shape), d[f"state_{cp}"]
        e_err, r_err = rel(eng, ext), rel(rgpu, ext)
        print(f"DNLS n={n} t={cp} ({form}): engine {e_err:.2e}, reference kernels {r_err:.2e} from the extended-precision "
              f"run; engine vs reference kernels {rel(eng, rgpu):.2e}")
        assert e_err <= 2 * r_err + 1e-14, f"t={cp}: the engine is less accurate than the reference kernels"
        if cp == 100:
            assert rel(eng, rgpu) <= STATE_TOL
        if cp == int(d["checkpoints"][-1]):
            en_e, en_r, en_x = O.energies(mdl, eng), O.energies(mdl, rgpu), O.energies(mdl, ext)
            drift_x = np.abs(en_x - e0).max()
            err_e, err_r = np.abs(en_e - en_x).max(), np.abs(en_r - en_x).max()
            print(f"   energy drift: engine {np.abs(en_e - e0).max():.3e}, reference kernels "
                  f"{np.abs(en_r - e0).max():.3e}, extended {drift_x:.3e}; energy error per chain against the "
                  f"extended run: engine {err_e:.3e}, reference kernels {err_r:.3e}")
            # the drift is mostly the splitting error itself (the extended-precision run has it too);
            # each chain's energy in double precision departs from its extended-precision energy by the
            # rounding of the whole run, and the engine's departure may be no larger than the
            # reference kernels' (the largest drift over the chains is not compared: a run can drift
            # less than the extended one)
            assert err_e <= max(2 * err_r, 1e-3 * drift_x)
    job.close()
    ctx.close()
    ref.close()


def test_ddnkg_configuration_full_run(gpu):
    """The dDNKG benchmark configuration (256 sites, masses U[1, 3], beta = 1, dt = 0.05) over its
    full 5 10^4 steps on 16 chains, sampled every 5000 steps."""
    torch = pytest.importorskip("torch")
    n, copies, dt, b, steps, every = 256, 16, 0.05, 100, 50000, 5000
    masses = ic.masses_uniform(n, seed=777)
    state = ic.ddnkg_ensemble(masses, copies, 0.5, 20, seed=12345)
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model("dDNKG", n, copies, dt, masses=masses, beta=1.0), b)
    job.upload(state)
    dev_o = O.Model("dDNKG", n, copies, dt, masses=masses, beta=1.0, order=O.ORDER_DEVICE)
    ref_o = O.Model("dDNKG", n, copies, dt, masses=masses, beta=1.0, order=O.ORDER_REFERENCE)
    eig = O.eigensystem(n, dev_o.mp2)
    ref = refgpu(256) if O.RefGPU.available(256) else None
    dev = torch.from_numpy(state.copy()).cuda() if ref else None
    od, orr = state.copy(), state.copy()
    e0 = O.energies(dev_o, state)
    for t in range(0, steps + 1, every):
        lin, wt, inf = job.linenergies()
        eng = job.download().reshape(state.shape)
        assert np.array_equal(eng, od), f"t={t}: not bit-identical to the oracle's device order"
        elin = O.linenergies(dev_o, od, eig)
        if t:   # at t = 0 unexcited modes sit at rounding level and WT is ill-conditioned
            check_diagnostics(lin, wt, inf, elin, False, f"dDNKG t={t}")
        if ref is not None:
            rg = dev.cpu().numpy().reshape(state.shape)
            assert np.array_equal(eng, rg), f"t={t}: not bit-identical to the reference's warp kernel"
        if t < steps:
            job.advance(every)
            od = O.advance(dev_o, od, every, b, order=O.ORDER_DEVICE).reshape(state.shape)
            orr = O.advance(ref_o, orr, every, b, order=O.ORDER_REFERENCE).reshape(state.shape)
            if ref is not None:
                ref.advance(ref_o, dev.data_ptr(), every, b)
    job.close()
    ctx.close()
    drift_e = np.abs(O.energies(dev_o, od) / e0 - 1).max()
    drift_r = np.abs(O.energies(ref_o, orr) / e0 - 1).max()
    print(f"dDNKG 5e4 steps: relative drift engine {drift_e:.3e}, reference CPU arithmetic {drift_r:.3e}")
    assert drift_e <= 1.1 * drift_r


@pytest.mark.parametrize("form", DNLS_FORMS)
def test_dnls_long_run_drift(gpu, form):
    """DNLS over 10^4 steps from a state with every mode excited (norm density 1): the engine's
    energy drift stays at or below the reference kernels'."""
    torch = pytest.importorskip("torch")
    ref = refgpu(64)
    n, copies, dt, b, steps = 64, 32, 0.01, 100, 10000
    psi = ic.dnls_ensemble(n, copies, 1.0, list(range(n)), seed=12345)
    state = np.ascontiguousarray(psi).view(np.float64).reshape(copies, n, 2)
    mdl = O.Model("DNLS", n, copies, dt, beta=1.0)
    eng, _, _ = engine_run(gpu, "DNLS", n, copies, dt, dict(beta=1.0, flags=DNLS_FORMS[form]), None, state, steps, b)
    dev = torch.from_numpy(state.copy()).cuda()
    ref.dnls_advance(mdl, dev.data_ptr(), steps, b)
    rg = dev.cpu().numpy().reshape(state.shape)
    ref.close()
    e0 = O.energies(mdl, state)
    drift_e = np.abs(O.energies(mdl, eng) - e0).max()
    drift_r = np.abs(O.energies(mdl, rg) - e0).max()
    print(f"DNLS n={n} 10^4 steps ({form}): energy drift engine {drift_e:.3e}, reference kernels {drift_r:.3e}")
    assert drift_e <= 1.1 * drift_r
