"""Integrator parity on the GPU, through the C ABI (nlc_job_* / nlc_move).

* Bit-exact against the oracle's device operation order (oracle/nlc_oracle.c move_chain_device):
  every FP64 operation of the kernels is an explicit round-to-nearest intrinsic and the table exp
  is replayed exactly, so the bytes must be identical for every model, variant and launch tier.
* Within 1e-12 (max-norm relative) of the reference CPU arithmetic after 10^3 steps, the
  tolerance the acceptance criteria set for the state.
"""
import os

import numpy as np
import pytest

import oracle as O
from nlchains_gb300 import ic

pytestmark = pytest.mark.gpu


def gpu_run(nlc, model, n, copies, dt, params, state, steps, batching, lanes=None, masses=None):
    old = os.environ.get("NLC_FORCE_LANES")
    if lanes:
        os.environ["NLC_FORCE_LANES"] = str(lanes)
    try:
        ctx = nlc.Context(0)
        job = ctx.job(nlc.Model(model, n, copies, dt, masses=masses, **params), batching)
        if lanes:
            assert job.ctx is ctx
        job.upload(state)
        job.advance(steps)
        out = job.download()
        job.close()
        ctx.close()
        return out
    finally:
        if lanes:
            if old is None:
                del os.environ["NLC_FORCE_LANES"]
            else:
                os.environ["NLC_FORCE_LANES"] = old


# (model, n, params, lanes per chain or None for the tuned shape)
CASES = [
    ("FPUT", 64, dict(alpha=0.0, beta=1.0), None),
    ("FPUT", 64, dict(alpha=0.0, beta=1.0), 32),
    ("FPUT", 64, dict(alpha=0.0, beta=1.0), 4),
    ("FPUT", 64, dict(alpha=0.25, beta=0.7), 16),
    ("FPUT", 2, dict(alpha=0.1, beta=1.0), None),
    ("FPUT", 5, dict(alpha=0.0, beta=1.0), 1),
    ("FPUT", 100, dict(alpha=0.3, beta=1.0), 8),
    ("FPUT", 1000, dict(alpha=0.0, beta=1.0), 64),
    ("DNKG", 128, dict(m=1.0, beta=1.0), None),
    ("DNKG", 128, dict(m=1.0, beta=1.0), 8),
    ("DNKG", 37, dict(m=0.5, beta=0.3), 4),
    ("DNKG", 3, dict(m=1.0, beta=1.0), 2),
    ("DNKG", 1000, dict(m=1.0, beta=1.0), 128),
    ("DNKG", 4000, dict(m=0.2, beta=0.5), 512),
    ("Toda", 128, dict(alpha=0.5), None),
    ("Toda", 128, dict(alpha=0.5), 32),
    ("Toda", 48, dict(alpha=0.8), 4),
    ("Toda", 2048, dict(alpha=0.5), 256),
    ("dDNKG", 256, dict(beta=1.0), None),
    ("dDNKG", 77, dict(beta=0.5), 8),
    ("dDNKG", 31, dict(beta=1.0), 2),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-n{c[1]}-G{c[3]}-{'-'.join(f'{k}{v}' for k, v in c[2].items())}")
def test_bit_exact_against_device_order_oracle(gpu, case):
    model, n, params, lanes = case
    copies = 13    # not a multiple of any group count: exercises the inert groups of the last unit
    dt = 0.05
    masses = ic.masses_uniform(n, seed=n) if model == "dDNKG" else None
    if model == "dDNKG":
        state = ic.ddnkg_ensemble(masses, copies, 0.5, max(1, n // 10), seed=5)
    else:
        m = params.get("m", 0.0)
        state = ic.real_ensemble(n, copies, 0.4, ic.low_modes(n, 0.1, include_zero=m > 0), m=m, seed=n)
    out = gpu_run(gpu, model, n, copies, dt, params, state, 30, 10, lanes=lanes, masses=masses)
    mdl = O.Model(model, n, copies, dt, masses=masses, **params)
    exp = O.advance(mdl, state, 30, 10, order=O.ORDER_DEVICE).reshape(copies, n, 2)
    if not np.array_equal(out, exp):
        diff = np.abs(out - exp)
        pytest.fail(f"not bit-exact: max abs diff {diff.max():.3e} at {np.unravel_index(diff.argmax(), diff.shape)}, "
                    f"{np.count_nonzero(diff)} elements differ")


REFERENCE_CASES = [
    # the FPUT-beta ensemble (N=64, dt=0.1, energy density 0.1 over k=+-1..4) and the DNKG / Toda
    # ensembles of 128 sites (dt=0.05, energy density 0.5 over the lowest 8% of the modes)
    ("FPUT", 64, dict(alpha=0.0, beta=1.0), 0.1, 0.1, dict(kmax=4, include_zero=False), 0.0),
    ("DNKG", 128, dict(m=1.0, beta=1.0), 0.05, 0.5, dict(fraction=0.08), 1.0),
    ("Toda", 128, dict(alpha=0.5), 0.05, 0.5, dict(fraction=0.08, include_zero=False), 0.0),
]


@pytest.mark.parametrize("case", REFERENCE_CASES, ids=lambda c: c[0])
def test_state_within_1e12_of_reference_arithmetic_after_1000_steps(gpu, case):
    model, n, params, dt, eps, modes, m = case
    copies = 16
    state = ic.real_ensemble(n, copies, eps, ic.low_modes(n, **modes), m=m, seed=21)
    out = gpu_run(gpu, model, n, copies, dt, params, state, 1000, 100)
    mdl = O.Model(model, n, copies, dt, **params)
    ref = O.advance(mdl, state, 1000, 100, order=O.ORDER_REFERENCE).reshape(copies, n, 2)
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()


def test_ddnkg_within_1e12_of_reference_arithmetic(gpu):
    n, copies = 256, 8
    masses = ic.masses_uniform(n, seed=9)
    state = ic.ddnkg_ensemble(masses, copies, 0.5, 20, seed=10)
    out = gpu_run(gpu, "dDNKG", n, copies, 0.05, dict(beta=1.0), state, 1000, 100, masses=masses)
    mdl = O.Model("dDNKG", n, copies, 0.05, beta=1.0, masses=masses)
    ref = O.advance(mdl, state, 1000, 100, order=O.ORDER_REFERENCE).reshape(copies, n, 2)
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()


def test_level1_operator_on_caller_memory_matches_job(gpu):
    """nlc_move on a caller-owned device buffer (torch allocation) gives the job path's bytes."""
    torch = pytest.importorskip("torch")
    n, copies = 64, 40
    state = ic.real_ensemble(n, copies, 0.1, ic.low_modes(n, kmax=4, include_zero=False), seed=3)
    model = gpu.Model("FPUT", n, copies, 0.1, alpha=0.0, beta=1.0)
    plan = gpu.Plan(model)
    dev = torch.from_numpy(state.copy()).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(3):
        plan.move(dev.data_ptr(), 10, stream)
    torch.cuda.synchronize()
    out = dev.cpu().numpy()
    exp = gpu_run(gpu, "FPUT", n, copies, 0.1, dict(alpha=0.0, beta=1.0), state, 30, 10)
    assert np.array_equal(out, exp)


def test_zero_steps_is_a_no_op(gpu):
    n, copies = 16, 4
    state = ic.real_ensemble(n, copies, 0.1, ic.low_modes(n, kmax=2, include_zero=False), seed=1)
    out = gpu_run(gpu, "FPUT", n, copies, 0.1, dict(alpha=0.0, beta=1.0), state, 0, 10)
    assert np.array_equal(out, state)


def test_pipelined_sampling_equals_synchronous(gpu):
    """Two result slots with the next batch enqueued before the previous sample is read give the
    same samples and states as the synchronous loop."""
    n, copies, b, rounds = 64, 96, 10, 6
    model = gpu.Model("FPUT", n, copies, 0.1, alpha=0.0, beta=1.0)
    state = ic.real_ensemble(n, copies, 0.1, ic.low_modes(n, kmax=4, include_zero=False), seed=5)
    ctx = gpu.Context(0)
    sync = ctx.job(model, b)
    sync.upload(state)
    exp = []
    for r in range(rounds):
        lin, wt, inf = sync.linenergies()
        exp.append((lin, wt, inf, sync.download()))
        sync.advance(b)
    pipe = ctx.job(model, b)
    pipe.upload(state)
    pipe.sample_async(0, copy_state=True)
    got = []
    for r in range(rounds):
        pipe.advance(b)
        pipe.sample_async((r + 1) % 2, copy_state=True)
        got.append(pipe.sample_wait(r % 2, with_state=True))
    for (el, ew, ei, es), (gl, gw, gi, gs) in zip(exp, got):
        assert np.array_equal(el, gl) and ew == gw and ei == gi and np.array_equal(es, gs)
    sync.close()
    pipe.close()
    ctx.close()


def test_two_jobs_taking_turns(gpu):
    """Two jobs alternating as a double-buffered end-to-end loop does (upload without waiting, the
    integration ordered after the other job's by nlc_job_after, sample, read back): every step's
    state and sample equal the synchronous single-job results; unknown job ids are rejected."""
    n, copies, b, rounds = 64, 4096, 20, 5
    model = gpu.Model("DNKG", n, copies, 0.05, m=1.0, beta=1.0)
    inputs = [0.3 * np.random.default_rng(10 + r).standard_normal((copies, n, 2)) for r in range(rounds)]
    ctx = gpu.Context(0)
    ref = ctx.job(model, b)
    exp = []
    for st in inputs:
        ref.upload(st)
        ref.advance(b)
        lin, wt, inf = ref.linenergies()
        exp.append((lin, wt, inf, ref.download()))
    jobs = [ctx.job(model, b) for _ in range(2)]
    ins = [np.ascontiguousarray(st) for st in inputs]
    got = []

    def issue(i):
        job = jobs[i % 2]
        job.upload(ins[i], wait=False)
        if i:
            job.after(jobs[(i - 1) % 2])
        job.advance(b)
        job.sample_async(0)

    issue(0)
    for i in range(rounds):
        if i + 1 < rounds:
            issue(i + 1)
        lin, wt, inf, _ = jobs[i % 2].sample_wait(0)
        got.append((lin, wt, inf, jobs[i % 2].download()))
    for (el, ew, ei, es), (gl, gw, gi, gs) in zip(exp, got):
        assert np.array_equal(el, gl) and ew == gw and ei == gi and np.array_equal(es, gs)
    with pytest.raises(gpu.NlcError) as e:
        gpu._check(gpu.lib().nlc_job_after(ctx._h, jobs[0].id, 987654321))
    assert e.value.code == gpu.ENOTFOUND
    for job in jobs + [ref]:
        job.close()
    ctx.close()


@pytest.mark.parametrize("name,n,params,window", [
    ("FPUT", 64, dict(alpha=0.0, beta=1.0), None),
    ("DNLS", 97, dict(beta=1.0), None),
    ("dDNKG", 256, dict(beta=1.0), None),      # tensor-core projection inside the graph
    ("DNKG", 600, dict(m=1.0, beta=1.0), 64),  # windowed tier: launches plus a device copy per batch
])
def test_graph_steps_equal_plain(gpu, name, n, params, window):
    """nlc_job_step_async (one CUDA graph launch per batch and sample) gives the same samples and
    states as nlc_job_advance + nlc_job_sample_async."""
    copies, b, rounds = 24, 7, 5
    masses = ic.masses_uniform(n, seed=4) if name == "dDNKG" else None
    state = 0.3 * np.random.default_rng(n).standard_normal((copies, n, 2))
    old = os.environ.get("NLC_FORCE_WINDOW")
    if window:
        os.environ["NLC_FORCE_WINDOW"] = str(window)
    try:
        ctx = gpu.Context(0)
        runs = []
        for graphs in (False, True):
            job = ctx.job(gpu.Model(name, n, copies, 0.01, masses=masses, **params), b)
            job.upload(state)
            job.sample_async(0, copy_state=True)
            got = []
            for r in range(rounds):
                if graphs:
                    job.step_async((r + 1) % 2, copy_state=True)
                else:
                    job.advance(b)
                    job.sample_async((r + 1) % 2, copy_state=True)
                got.append(job.sample_wait(r % 2, with_state=True))
            got.append(job.sample_wait(rounds % 2, with_state=True))
            runs.append(got)
            job.close()
        ctx.close()
    finally:
        if window:
            if old is None:
                del os.environ["NLC_FORCE_WINDOW"]
            else:
                os.environ["NLC_FORCE_WINDOW"] = old
    for (pl, pw, pi, ps), (gl, gw, gi, gs) in zip(*runs):
        assert np.array_equal(pl, gl) and pw == gw and pi == gi and np.array_equal(ps, gs)


@pytest.mark.parametrize("name,params,m,steps,copies", [
    ("DNKG", dict(m=1.0, beta=1.0), 1.0, 100000, 64),
    ("Toda", dict(alpha=0.5), 0.0, 20000, 32),
], ids=["DNKG", "Toda"])
def test_long_run_bit_exact_and_drift(gpu, name, params, m, steps, copies):
    """A long run of the benchmark configuration (N = 128, dt = 0.05; DNKG m = beta = 1 for 10^5
    steps, Toda alpha = 0.5 for 2 10^4; a low-mode state at energy density 0.5): the state stays
    bit-identical to the oracle's device operation order through the whole run (the dynamics is
    chaotic, so a single differing bit would grow), and the energy drift is no larger than that of
    the reference's arithmetic order."""
    n, b = 128, 100
    state = ic.real_ensemble(n, copies, 0.5, ic.low_modes(n, 0.08, include_zero=m > 0), m=m, seed=11)
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model(name, n, copies, 0.05, **params), b)
    job.upload(state)
    job.advance(steps)
    out = job.download().reshape(copies, n, 2)
    e_gpu = job.energies()
    job.close()
    ctx.close()
    mdl = O.Model(name, n, copies, 0.05, **params)
    dev = O.advance(mdl, state, steps, b, order=O.ORDER_DEVICE).reshape(copies, n, 2)
    assert np.array_equal(out, dev)
    ref = O.advance(mdl, state, steps, b, order=O.ORDER_REFERENCE).reshape(copies, n, 2)
    e0 = O.energies(mdl, state)
    drift_gpu = np.abs(e_gpu / e0 - 1).max()
    drift_ref = np.abs(O.energies(mdl, ref) / e0 - 1).max()
    assert drift_gpu <= 2 * drift_ref + 1e-12, (drift_gpu, drift_ref)


def test_fput_benchmark_configuration_full_run(gpu):
    """The FPUT-beta benchmark configuration in full (N = 64, 1024 copies, alpha = 0, beta = 1,
    dt = 0.1, 10^4 steps sampled every 100: 101 samples; energy density 0.1 in modes +-1..+-4)
    against the oracle: the final state bit-identical, the linear energies of every sample within
    1e-10 of the largest and the information entropy within 1e-10.  (The WT entropy, a sum of logs
    of mode energies, is ill-conditioned while modes hold rounding-level energy, as here.)"""
    n, copies, b, steps, dt = 64, 1024, 100, 10000, 0.1
    state = ic.real_ensemble(n, copies, 0.1, ic.low_modes(n, kmax=4, include_zero=False), seed=21)
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model("FPUT", n, copies, dt, alpha=0.0, beta=1.0), b)
    job.upload(state)
    mdl = O.Model("FPUT", n, copies, dt, alpha=0.0, beta=1.0)
    cur = state
    for t in range(0, steps + 1, b):
        if t:
            job.advance(b)
            cur = O.advance(mdl, cur, b, b, order=O.ORDER_DEVICE)
        lin, wt, inf = job.linenergies()
        elin = O.linenergies(mdl, cur)
        _, einf = O.entropies(elin, True)
        assert np.abs(lin - elin).max() <= 1e-10 * elin.max(), t
        assert abs(inf - einf) <= 1e-10 * max(1.0, abs(einf)), t
    assert np.array_equal(job.download().reshape(copies, n, 2), cur.reshape(copies, n, 2))
    job.close()
    ctx.close()


@pytest.mark.parametrize("name,n,params,masses_seed", [
    ("FPUT", 64, dict(alpha=0.0, beta=1.0), None),
    ("FPUT", 37, dict(alpha=0.3, beta=0.8), None),
    ("DNKG", 48, dict(m=0.5, beta=1.0), None),
    ("Toda", 40, dict(alpha=0.5), None),
    ("dDNKG", 33, dict(beta=1.0), 5),
])
def test_fused_rounds_equal_one_launch_per_round(gpu, name, n, params, masses_seed):
    """Job.advance over several rounds of kernel_batching steps with no sample in between fuses rounds
    into fewer launches (each round still closed by its own final drift and the next opened unmerged):
    the result is bit-identical to one launch per round (the oracle's launches of `batching` steps),
    and for a small ensemble the launch count drops."""
    copies, b, rounds = 96, 10, 30
    masses = ic.masses_uniform(n, seed=masses_seed) if masses_seed is not None else None
    rng = np.random.default_rng(n)
    state = rng.standard_normal((copies, n, 2)) * 0.3
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model(name, n, copies, 0.05, masses=masses, **params), b)
    job.upload(state)
    before = gpu.kernel_launches()
    job.advance(b * rounds)
    job.wait()
    launches = gpu.kernel_launches() - before
    out = job.download()
    job.close()
    ctx.close()
    mdl = O.Model(name, n, copies, 0.05, masses=masses, **params)
    exp = O.advance(mdl, state, b * rounds, b, order=O.ORDER_DEVICE).reshape(copies, n, 2)
    assert np.array_equal(out, exp)
    assert launches < rounds, f"{launches} launches for {rounds} rounds: no rounds were fused"
