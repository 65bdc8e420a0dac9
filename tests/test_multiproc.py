"""Multi-rank host logic on CPU (gloo, world size 2): permutation shards
cover every iteration once, the JS gather reassembles them in order, and the
beta fit on rank 0 equals the single-process one.  The per-shard compute is
the oracle (no GPU here)."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import sys
    sys.path[:0] = [os.path.join(ROOT, "eddy-gpu_gb300"), os.path.join(ROOT, "oracle")]
    import torch.distributed as dist

    import oracle as O
    from eddy_gpu import distributed as D
    from eddy_gpu import synth
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w = synth.make(2, seed=0)
    name, genes, prior = w.sets[0]
    R = 9
    labs = O.counter_labels(3, 0, w.labels, R)
    prm = O.params(mp=3, pw=0.5)

    def compute(first, count):
        return O.units(w.data[genes], labs[first:first + count], prior, prm, threads=1)

    js = D.sharded_permutation_test(compute, R, world, rank)
    if rank == 0:
        np.save(out, js)
    dist.destroy_process_group()


def test_shard_ranges():
    from eddy_gpu.distributed import shard
    for count in (0, 1, 7, 100):
        for world in (1, 2, 3, 8):
            got = []
            for r in range(world):
                s, c = shard(1, count, world, r)
                got.extend(range(s, s + c))
            assert got == list(range(1, 1 + count))


def test_two_rank_gather_and_beta_fit(tmp_path, oracle_lib):
    out = str(tmp_path / "js.npy")
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    js = np.load(out)
    from eddy_gpu import synth
    w = synth.make(2, seed=0)
    name, genes, prior = w.sets[0]
    labs = oracle_lib.counter_labels(3, 0, w.labels, 9)
    ref, _ = oracle_lib.units(w.data[genes], labs, prior, oracle_lib.params(mp=3, pw=0.5))
    assert np.array_equal(js, ref)
    assert oracle_lib.pddn(js)[3] == oracle_lib.pddn(ref)[3]
