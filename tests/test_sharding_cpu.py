"""Chains sharded over ranks (the multi-GPU path), exercised as two gloo
processes on the CPU: the per-rank ESS and moment summaries combine into
the figures of all chains together."""
import json
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_data(rank):
    rng = np.random.default_rng(100 + rank)
    samples = rng.normal(loc=rank, scale=1.0 + rank, size=(50 + 30 * rank, 7))
    ess = rng.uniform(10, 20, size=7)
    return samples, ess, 1.5 + rank


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist

    from hmclab_gb300 import sharding

    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        r, w, lr = sharding.rank_environment()
        samples, ess, sec = _rank_data(rank)
        tot, tmax = sharding.combine_ess(ess, sec)
        m, s = sharding.combine_moments(samples.mean(axis=0), samples.std(axis=0), samples.shape[0])
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"env": [r, w, lr], "ess": tot.tolist(), "tmax": tmax, "mean": m.tolist(), "std": s.tolist(),
                       "seed": sharding.rank_seed(7, rank)}, f)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_combine_summaries(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    data = [_rank_data(r) for r in range(world)]
    allx = np.concatenate([d[0] for d in data])
    for r, out in enumerate(res):
        assert out["env"] == [r, world, r]
        np.testing.assert_allclose(out["ess"], data[0][1] + data[1][1], rtol=1e-12)
        assert out["tmax"] == 2.5
        np.testing.assert_allclose(out["mean"], allx.mean(axis=0), rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(out["std"], allx.std(axis=0), rtol=1e-10)
    assert res[0]["seed"] != res[1]["seed"]


def test_single_process_without_a_group():
    from hmclab_gb300 import sharding

    ess, t = sharding.combine_ess(np.array([3.0, 4.0]), 2.0)
    np.testing.assert_array_equal(ess, [3.0, 4.0])
    assert t == 2.0
    m, s = sharding.combine_moments(np.array([1.0]), np.array([2.0]), 10)
    assert m[0] == 1.0 and abs(s[0] - 2.0) < 1e-12
