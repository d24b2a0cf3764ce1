"""The continuous-batching request server (nlc_server_*): every result equals the same request run
alone through the job API, whatever else was in the mix, and admission respects the HBM budget."""
import numpy as np
import pytest

from nlchains_gb300 import ic

pytestmark = pytest.mark.gpu


def make_state(model, n, copies, seed, masses=None):
    if model == "DNLS":
        psi = ic.dnls_ensemble(n, copies, 1.0, ic.low_modes(n, 0.2), seed=seed)
        return np.ascontiguousarray(psi).view(np.float64).reshape(copies, n, 2)
    if model == "dDNKG":
        return ic.ddnkg_ensemble(masses, copies, 0.3, max(2, n // 8), seed=seed)
    return 0.3 * np.random.default_rng(seed).standard_normal((copies, n, 2))


# (model, n, copies, b, steps, params): repeated shapes share a batched launch
MIX = [
    ("FPUT", 64, 200, 10, 50, dict(alpha=0.0, beta=1.0)),
    ("FPUT", 64, 77, 10, 30, dict(alpha=0.0, beta=1.0)),
    ("FPUT", 64, 33, 20, 40, dict(alpha=0.0, beta=1.0)),
    ("FPUT", 60, 45, 10, 20, dict(alpha=0.0, beta=1.0)),
    ("Toda", 128, 50, 10, 20, dict(alpha=0.5)),
    ("Toda", 128, 51, 10, 30, dict(alpha=0.5)),
    ("DNKG", 100, 64, 10, 20, dict(m=1.0, beta=1.0)),
    ("DNKG", 100, 64, 10, 20, dict(m=1.0, beta=0.5)),
    ("dDNKG", 48, 40, 10, 20, dict(beta=1.0)),
    ("dDNKG", 48, 41, 10, 30, dict(beta=1.0)),
    ("DNLS", 128, 30, 5, 10, dict(beta=1.0)),
    ("DNLS", 62, 40, 5, 10, dict(beta=1.0)),      # the stencil form on 4 lanes of a warp
    ("DNLS", 5000, 3, 5, 10, dict(beta=1.0)),     # the stencil form in windows (tier 6)
]


def alone(nlc, model, b, steps, state):
    ctx = nlc.Context(0)
    job = ctx.job(model, b)
    job.upload(state)
    ents = []
    for t in range(0, steps + 1, b):
        if t:
            job.advance(b)
        lin, wt, inf = job.linenergies()
        ents.append((wt, inf))
    out = job.download()
    job.close()
    ctx.close()
    return out, lin, np.array(ents)


def run_mix(nlc, mix, **server_kw):
    srv = nlc.Server(0, **server_kw)
    reqs = []
    for i, (name, n, copies, b, steps, params) in enumerate(mix):
        masses = ic.masses_uniform(n, seed=100 + i) if name == "dDNKG" else None
        model = nlc.Model(name, n, copies, 0.05, masses=masses, **params)
        state = make_state(name, n, copies, seed=i, masses=masses)
        reqs.append((srv.submit(model, b, steps, state), model, b, steps, state))
    results = []
    for rid, model, b, steps, state in reqs:
        srv.wait(rid, 120000)
        st = srv.poll(rid)
        results.append((st,) + srv.result(rid))
    srv.close()
    return reqs, results


def test_mixed_results_equal_alone(gpu):
    reqs, results = run_mix(gpu, MIX)
    for (rid, model, b, steps, state), (st, fstate, flin, ents, rc) in zip(reqs, results):
        assert rc == gpu.OK and st["state"] == gpu.REQ_DONE and st["steps_done"] == steps
        out, lin, aents = alone(gpu, model, b, steps, state)
        assert np.array_equal(fstate, out), f"{model.name} n={model.chain_length}: state differs from the run alone"
        assert ents.shape == aents.shape
        # the server's diagnostics use fewer partial rows: equal to rounding
        assert np.abs(flin - lin).max() <= 1e-12 * np.abs(lin).max()
        assert np.abs(ents - aents).max() <= 1e-10 * max(1.0, np.abs(aents).max())
        assert st["submit_ms"] <= st["start_ms"] <= st["finish_ms"]


@pytest.mark.parametrize("quantum_ms", [1e-6, -1.0])
def test_segmented_rounds_equal_alone(gpu, quantum_ms):
    # 1e-6 ms: every round is integrated one step per launch (open segments, merged drift between
    # them); -1: every round in one launch.  Both equal the run alone bit for bit.
    reqs, results = run_mix(gpu, MIX, quantum_ms=quantum_ms)
    for (rid, model, b, steps, state), (st, fstate, flin, ents, rc) in zip(reqs, results):
        assert rc == gpu.OK and st["steps_done"] == steps and len(ents) == steps // b + 1
        out, lin, aents = alone(gpu, model, b, steps, state)
        assert np.array_equal(fstate, out), f"{model.name} n={model.chain_length}: segmented run differs"
        assert np.abs(ents - aents).max() <= 1e-10 * max(1.0, np.abs(aents).max())


def test_budget_admission_serialises(gpu):
    # a budget of one byte admits one request at a time (a request larger than the budget runs
    # alone when nothing else is active); all still complete with the same results
    mix = MIX[:3] + MIX[4:6]
    reqs, results = run_mix(gpu, mix, hbm_budget_bytes=1)
    spans = sorted((st["start_ms"], st["finish_ms"]) for st, *_ in results)
    for (s0, f0), (s1, f1) in zip(spans, spans[1:]):
        assert s1 >= f0 - 1e-6, "requests overlapped under a one-byte budget"
    for (rid, model, b, steps, state), (st, fstate, flin, ents, rc) in zip(reqs, results):
        out, lin, aents = alone(gpu, model, b, steps, state)
        assert np.array_equal(fstate, out)


def test_blowup_fails_only_that_request(gpu):
    srv = gpu.Server(0)
    good = gpu.Model("FPUT", 32, 16, 0.05, alpha=0.0, beta=1.0)
    bad_state = np.zeros((16, 32, 2))
    bad_state[3, 4, 0] = np.nan
    r_bad = srv.submit(good, 10, 50, bad_state)
    state = make_state("FPUT", 32, 16, seed=5)
    r_good = srv.submit(good, 10, 50, state)
    srv.wait(r_bad, 60000)
    srv.wait(r_good, 60000)
    assert srv.poll(r_bad)["state"] == gpu.REQ_FAILED and srv.poll(r_bad)["error"] == gpu.EBLOWUP
    assert srv.poll(r_good)["state"] == gpu.REQ_DONE
    _, _, _, rc = srv.result(r_bad)
    assert rc == gpu.EBLOWUP
    fstate, _, _, rc = srv.result(r_good)
    assert rc == gpu.OK
    out, _, _ = alone(gpu, good, 10, 50, state)
    assert np.array_equal(fstate, out)
    srv.close()


def test_wait_times_out_then_completes(gpu):
    srv = gpu.Server(0)
    model = gpu.Model("Toda", 1024, 2048, 0.05, alpha=0.5)
    rid = srv.submit(model, 100, 3000, make_state("Toda", 1024, 2048, seed=9))
    with pytest.raises(gpu.NlcError) as e:
        srv.wait(rid, 0)
    assert e.value.code == gpu.ETIMEDOUT
    srv.wait(rid, 300000)
    assert srv.poll(rid)["state"] == gpu.REQ_DONE
    srv.close()
