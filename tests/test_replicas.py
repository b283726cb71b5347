"""Replica sharding across ranks, world size 2 on the gloo backend (CPU):
each rank phases its own chunk with the CPU oracle, ranks agree on the
max elapsed time, and the chunks and random streams differ by rank."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_dir):
    import sys
    import time
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "oracle")]
    import oracle as O
    from glphase_gb300 import replicas, synth
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rp = replicas.plan(12, rank=rank, world=world)
    w = synth.Workload("rep", N=10, S=130, founders=5, depth=3, burnin=1, sampling=1,
                       cycles=6, seed=rp.data_seed)
    m, haps = synth.initial_state(synth.generate(w), seed=rp.data_seed)
    quad, props = synth.uniform_proposals(m.N, haps.shape[0], 6,
                                          np.random.default_rng(rp.data_seed))
    pb = O.OracleProblem(haps, m.emit, m.t, m.tran, m.pc, 6)
    dist.barrier()
    t0 = time.perf_counter()
    q, h, like = O.generation(pb, pb.trace(seed=rp.rng_seed, generation=0), quad, props, 1.0,
                              like=True, nthreads=1)
    el = time.perf_counter() - t0 + 0.01 * rank
    mx = replicas.max_elapsed(el)
    np.savez(os.path.join(out_dir, f"r{rank}.npz"), like=like, mx=mx, el=el,
             seed=rp.rng_seed, data_seed=rp.data_seed)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    r0, r1 = (np.load(tmp_path / f"r{i}.npz") for i in range(2))
    assert float(r0["mx"]) == float(r1["mx"]) == max(float(r0["el"]), float(r1["el"]))
    assert int(r0["data_seed"]) != int(r1["data_seed"])
    assert int(r0["seed"]) != int(r1["seed"])
    assert not np.array_equal(r0["like"], r1["like"])


def test_plan_validates_rank():
    from glphase_gb300 import replicas
    with pytest.raises(ValueError):
        replicas.plan(1, rank=2, world=2)
    rp = replicas.plan(5, rank=1, world=4, local_rank=1)
    assert rp.data_seed == 1005 and rp.world == 4
