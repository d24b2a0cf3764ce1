"""The drop-in `nlchains` command line end to end on the GPU (files in the reference formats)."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from nlchains_gb300 import ic

pytestmark = pytest.mark.gpu


def run_cli(nlc, args, cwd):
    nlc.build()
    return subprocess.run([nlc.EXECUTABLE_PATH, *args], cwd=cwd, capture_output=True, text=True, timeout=300)


def test_fput_run_writes_reference_files(gpu, tmp_path):
    n, copies, b, steps, dt = 64, 32, 10, 50, 0.1
    # every mode excited: the WT entropy (sum of log e_k) is only well conditioned without empty modes
    state = 0.3 * np.random.default_rng(1).standard_normal((copies, n, 2))
    ic.write_state(tmp_path / "init", state)
    r = run_cli(gpu, ["FPUT", "-i", "init", "-n", str(n), "-c", str(copies), "--dt", str(dt), "-b", str(b),
                      "-s", str(steps), "-p", "out", "--alpha", "0", "--beta", "1", "--dump_interval", "20"], tmp_path)
    assert r.returncode == 0, r.stderr
    mdl = O.Model("FPUT", n, copies, dt, alpha=0.0, beta=1.0)
    ent = np.fromfile(tmp_path / "out-entropy").reshape(-1, 3)
    assert ent.shape == (steps // b + 1, 3)
    cur = state
    for i, t in enumerate(range(0, steps + 1, b)):
        if t:
            cur = O.advance(mdl, cur, b, b)
        lin = O.linenergies(mdl, cur)
        wt, inf = O.entropies(lin, True)
        assert ent[i, 0] == t * dt
        assert abs(ent[i, 1] - wt) < 1e-10 * max(1, abs(wt)) and abs(ent[i, 2] - inf) < 1e-10 * max(1, abs(inf))
        if t % 20 == 0 or t == steps:
            got = np.fromfile(tmp_path / f"out-linenergies-{t}")
            assert np.abs(got - lin).max() <= 1e-10 * lin.max()
            dump = np.fromfile(tmp_path / f"out-{t}").reshape(copies, n, 2)
            assert np.array_equal(dump, cur.reshape(copies, n, 2))
        else:
            assert not os.path.exists(tmp_path / f"out-{t}")


def test_ddnkg_writes_eigensystem(gpu, tmp_path):
    n, copies = 16, 8
    masses = ic.masses_uniform(n, seed=2)
    masses.tofile(tmp_path / "m")
    state = ic.ddnkg_ensemble(masses, copies, 0.3, 4, seed=3)
    ic.write_state(tmp_path / "init", state)
    r = run_cli(gpu, ["dDNKG", "-i", "init", "-n", str(n), "-c", str(copies), "--dt", "0.05", "-b", "10",
                      "-s", "20", "-p", "o", "-m", "m", "--beta", "1"], tmp_path)
    assert r.returncode == 0, r.stderr
    om = np.fromfile(tmp_path / "o-omegas")
    vec = np.fromfile(tmp_path / "o-eigenvectors").reshape(n, n)
    eom, evec = O.eigensystem(n, masses + 2)
    assert np.abs(om - eom).max() < 1e-12
    evec = evec.reshape(n, n)
    for k in range(n):
        assert min(np.abs(vec[k] - evec[k]).max(), np.abs(vec[k] + evec[k]).max()) < 1e-10


def test_entropy_limit_stops_early(gpu, tmp_path):
    n, copies = 32, 8
    state = ic.real_ensemble(n, copies, 0.1, ic.low_modes(n, kmax=2, include_zero=False), seed=4)
    ic.write_state(tmp_path / "init", state)
    # the initial information entropy is far above 0, so a limit above it stops at t = 0
    r = run_cli(gpu, ["FPUT", "-i", "init", "-n", str(n), "-c", str(copies), "--dt", "0.1", "-b", "10",
                      "-s", "0", "-p", "o", "--alpha", "0", "--beta", "1", "-e", "1e9"], tmp_path)
    assert r.returncode == 0, r.stderr
    ent = np.fromfile(tmp_path / "o-entropy").reshape(-1, 3)
    # the reference stops at its main loop's step, up to two batches past the sample that asked
    # (loop_control.hpp); the engine keeps one batch in flight, so it stops at t = 0 or t = 10
    assert 1 <= ent.shape[0] <= 3
    assert os.path.exists(tmp_path / "o-0")
    assert os.path.exists(tmp_path / f"o-{10 * (ent.shape[0] - 1)}")


CLI_MODELS = [
    ("DNKG", ["-m", "0.5", "--beta", "0.7"], dict(m=0.5, beta=0.7), 0.05),
    ("FPUT", ["--alpha", "0.3", "--beta", "0.8"], dict(alpha=0.3, beta=0.8), 0.05),
    ("Toda", ["--alpha", "0.5"], dict(alpha=0.5), 0.05),
    ("dDNKG", ["-m", "masses", "--beta", "1"], dict(beta=1.0), 0.05),
    ("DNLS", ["--beta", "1"], dict(beta=1.0), 0.01),
]


@pytest.mark.parametrize("name,flags,params,dt", CLI_MODELS, ids=[c[0] for c in CLI_MODELS])
@pytest.mark.parametrize("offset", [0, 20])
def test_every_model_matches_job_api(gpu, tmp_path, name, flags, params, dt, offset):
    """`nlchains <model>` against the job API on the same input: the entropy rows (times offset,
    offset + b, ..., steps), the linear energies of every dump and the final dump, identical (the
    same kernels run in both)."""
    n, copies, b, steps = 48, 24, 10, 60
    rng = np.random.default_rng(sum(map(ord, name)))
    state = 0.3 * rng.standard_normal((copies, n, 2))
    masses = ic.masses_uniform(n, seed=7) if name == "dDNKG" else None
    if masses is not None:
        masses.tofile(tmp_path / "masses")
    ic.write_state(tmp_path / "init", state)
    r = run_cli(gpu, [name, "-i", "init", "-n", str(n), "-c", str(copies), "--dt", str(dt), "-b", str(b), "-s", str(steps),
                      "-o", str(offset), "-p", "out", "--dump_interval", "20", *flags], tmp_path)
    assert r.returncode == 0, r.stderr
    ent = np.fromfile(tmp_path / "out-entropy").reshape(-1, 3)
    times = list(range(offset, steps + 1, b))
    assert ent.shape == (len(times), 3)
    ctx = gpu.Context(0)
    job = ctx.job(gpu.Model(name, n, copies, dt, masses=masses, **params), b)
    job.upload(state)
    for i, t in enumerate(times):
        if i:
            job.advance(b)
        lin, wt, inf = job.linenergies()
        assert ent[i, 0] == t * dt and ent[i, 1] == wt and ent[i, 2] == inf, (t, ent[i], wt, inf)
        if t % 20 == 0:
            assert np.array_equal(np.fromfile(tmp_path / f"out-linenergies-{t}"), lin)
            assert np.array_equal(np.fromfile(tmp_path / f"out-{t}").reshape(copies, n, 2),
                                  job.download().reshape(copies, n, 2))
    job.close()
    ctx.close()


def test_sigint_stops_an_endless_run(gpu, tmp_path):
    """`-s 0` runs until stopped (main.cpp:63); SIGINT stops it gracefully after the sample in flight
    (main.cpp:144, loop_control.hpp:22-25): exit status 0, one entropy row per sample at 0, b, 2b,
    ..., and a final dump at the last sample's step."""
    import signal
    import time
    n, copies, b, dt = 64, 256, 100, 0.05
    state = 0.3 * np.random.default_rng(6).standard_normal((copies, n, 2))
    ic.write_state(tmp_path / "init", state)
    gpu.build()
    p = subprocess.Popen([gpu.EXECUTABLE_PATH, "FPUT", "-i", "init", "-n", str(n), "-c", str(copies), "--dt", str(dt),
                          "-b", str(b), "-s", "0", "-p", "o", "--alpha", "0", "--beta", "1", "--dump_interval", "1000000"],
                         cwd=tmp_path, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    ent = tmp_path / "o-entropy"
    try:
        deadline = time.time() + 120
        while time.time() < deadline and not (ent.exists() and ent.stat().st_size >= 5 * 24):
            time.sleep(0.05)
        p.send_signal(signal.SIGINT)
        _, err = p.communicate(timeout=120)
    finally:
        if p.poll() is None:
            p.kill()
            p.wait()
    assert p.returncode == 0, err
    rows = np.fromfile(ent).reshape(-1, 3)
    assert rows.shape[0] >= 5
    steps = np.rint(rows[:, 0] / dt).astype(np.int64)
    assert np.array_equal(steps, b * np.arange(rows.shape[0]))
    assert np.all(np.isfinite(rows[:, 1:]))
    assert os.path.exists(tmp_path / "o-0")
    last = np.fromfile(tmp_path / f"o-{steps[-1]}").reshape(copies, n, 2)
    assert np.all(np.isfinite(last))
