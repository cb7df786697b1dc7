"""Replica (one process per GPU) host logic on CPU ranks with the gloo
backend, world size 2: barrier, maximum of the ranks' times, job sharding,
and the whole-job throughput the bench reports for N > 1. Each rank also
runs the CPU oracle on its shard of geometries to show that ranks work
independently and the union of shards is the full job."""

import json
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from fastercap_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import sys
    import torch.distributed as dist
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "oracle"))
    sys.path.insert(0, here)
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, lr = replicas.dist_env()
    assert (r, w, lr) == (rank, world, rank)
    replicas.barrier(w)
    # per-rank "times": the maximum must come back to every rank
    times = [1.0 + rank, 5.0 - rank]
    mx = replicas.max_over_ranks(times, w)
    # each rank solves its shard of the golden geometries with the oracle
    from conftest import golden_names, load_golden, model_arrays, solve_params, super_dim
    from pyoracle import Oracle
    names = golden_names()
    mine = replicas.shard(len(names), r, w)
    caps = {}
    for j in mine:
        g = load_golden(names[j])
        o = Oracle(model_arrays(g))
        o.fill()
        tol, pc = solve_params(g)
        cap, _, _, _ = o.solve(tol, pc, super_dim=super_dim(g))
        caps[names[j]] = cap.tolist()
    total = replicas.sum_over_ranks([len(mine)], w)[0]
    gathered = replicas.gather_to_all({"rank": r, "jobs": mine}, w)
    assert [x["rank"] for x in gathered] == list(range(w))
    assert sorted(j for x in gathered for j in x["jobs"]) == list(range(len(names)))
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
        json.dump({"max": mx, "mine": mine, "total": total, "caps": caps,
                   "value": replicas.throughput(3, w, mx[0])}, f)
    dist.destroy_process_group()


def test_gloo_two_ranks(tmp_path):
    world, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, start_method="spawn", join=True)
    res = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(world)]
    for d in res:
        assert d["max"] == [2.0, 5.0]
        assert d["value"] == pytest.approx(2 * 3 / 2.0)
    from conftest import golden_names, load_golden
    names = golden_names()
    assert sorted(res[0]["mine"] + res[1]["mine"]) == list(range(len(names)))
    assert not set(res[0]["mine"]) & set(res[1]["mine"])
    assert res[0]["total"] == len(names)
    # every geometry solved on some rank, and the rank's result is the reference's
    for d in res:
        for name, cap in d["caps"].items():
            ref = load_golden(name)["ref_cap"]
            np.testing.assert_allclose(np.array(cap), ref, rtol=1e-9)


def test_shard_and_throughput_single():
    assert replicas.shard(5, 0, 1) == [0, 1, 2, 3, 4]
    assert replicas.shard(5, 1, 2) == [1, 3]
    assert replicas.max_over_ranks([3.0], 1) == [3.0]
    assert replicas.throughput(10, 1, 2.0) == 5.0
