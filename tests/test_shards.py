"""Copies sharded over two processes (gloo, host only): the combined linear energies and entropies
equal those of the whole ensemble in one process, and the host entropies match the oracle."""
import os
import socket

import numpy as np
import pytest

import oracle as O


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, model_args, state, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    from nlchains_gb300 import Model, shards
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        name, n, copies, params = model_args
        first, count = shards.shard_range(copies, rank, world)
        local = O.Model(name, n, count, 0.05, **params)
        lin_local = O.linenergies(local, state[first:first + count])
        lin, wt, inf = shards.sample(lin_local, count, copies, Model(name, n, copies, 0.05, **params).a0is0)
        np.save(os.path.join(out_dir, f"rank{rank}.npy"), np.concatenate([lin, [wt, inf]]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name,params", [("FPUT", dict(alpha=0.0, beta=1.0)), ("DNKG", dict(m=1.0, beta=1.0)),
                                         ("DNLS", dict(beta=1.0))])
def test_two_process_combine_equals_one_process(tmp_path, name, params):
    mp = pytest.importorskip("torch.multiprocessing")
    n, copies, world = 48, 26, 2
    state = np.random.default_rng(11).standard_normal((copies, n, 2))
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, (name, n, copies, params), state, str(tmp_path)))
             for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    whole = O.Model(name, n, copies, 0.05, **params)
    exp_lin = O.linenergies(whole, state)
    exp_wt, exp_inf = O.entropies(exp_lin, O.a0is0(whole))
    for r in range(world):
        got = np.load(tmp_path / f"rank{r}.npy")
        assert np.abs(got[:n] - exp_lin).max() <= 1e-13 * np.abs(exp_lin).max()
        assert abs(got[n] - exp_wt) <= 1e-11 * max(1.0, abs(exp_wt))
        assert abs(got[n + 1] - exp_inf) <= 1e-11 * max(1.0, abs(exp_inf))


def test_shard_range_rejects_uneven_split():
    from nlchains_gb300 import shards
    assert shards.shard_range(12, 1, 3) == (4, 4)
    with pytest.raises(ValueError):
        shards.shard_range(10, 0, 3)


def test_host_entropies_match_oracle():
    import nlchains_gb300 as nlc
    rng = np.random.default_rng(3)
    lin = rng.random(64) + 0.01
    mask = (rng.random(64) < 0.5).astype(np.uint8)
    for a0 in (False, True):
        for m in (None, mask):
            wt, inf = nlc.entropies(lin, a0, m)
            ewt, einf = O.entropies(lin, a0, m)
            assert abs(wt - ewt) <= 1e-12 * max(1.0, abs(ewt)) and abs(inf - einf) <= 1e-12 * max(1.0, abs(einf))
    bad = lin.copy()
    bad[5] = 0.0   # log 0: non-finite WT, the reference's quit condition
    with pytest.raises(nlc.NlcError) as e:
        nlc.entropies(bad, False)
    assert e.value.code == nlc.EBLOWUP
