"""World-size-2 gloo runs on the CPU of the multi-rank host logic (mpm_gb300.distributed):
scene sharding covers every scene once, the timing collectives give the slowest rank, and
the whole-job rate of replicas and of sharded batches."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import json

    import torch.distributed as dist

    from mpm_gb300 import distributed as D
    from mpm_gb300 import scenes

    w, r, _ = D.init("gloo")
    assert (w, r) == (world, rank)
    all_scenes = scenes.config_batched(nscenes=9, seed=1)
    mine = D.shard(all_scenes, r, w)
    n_mine = sum(len(s["state"]["x"]) for s in mine)
    n_all = D.sum_over_ranks(n_mine)
    D.barrier()
    t_slowest = D.max_over_ranks(1.0 + r)  # rank r "took" 1 + r seconds
    res = {"rank": r, "scene_ids": [all_scenes.index(s) for s in mine], "n_all": n_all,
           "n_expected": sum(len(s["state"]["x"]) for s in all_scenes), "t_slowest": t_slowest,
           "replica_rate": D.job_rate(w * 1000 * 10, t_slowest), "batch_rate": D.job_rate(n_all * 50, t_slowest)}
    with open(os.path.join(out_dir, f"rank{r}.json"), "w") as f:
        json.dump(res, f)
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    import json

    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    ids = sorted(i for r in res for i in r["scene_ids"])
    assert ids == list(range(9))                        # every scene exactly once
    assert res[0]["scene_ids"] == [0, 2, 4, 6, 8] and res[1]["scene_ids"] == [1, 3, 5, 7]
    for r in res:
        assert r["n_all"] == r["n_expected"]            # the shards add up to the whole batch
        assert r["t_slowest"] == 2.0                    # max over ranks
        assert r["replica_rate"] == 2 * 1000 * 10 / 2.0
        assert r["batch_rate"] == r["n_expected"] * 50 / 2.0


def test_single_rank_and_bad_arguments():
    from mpm_gb300 import distributed as D

    assert D.shard(list(range(5)), 0, 1) == list(range(5))
    assert D.max_over_ranks(3.5) == 3.5 and D.sum_over_ranks(2.0) == 2.0
    with pytest.raises(ValueError):
        D.shard([1, 2], 2, 2)
    with pytest.raises(ValueError):
        D.job_rate(10, 0.0)
