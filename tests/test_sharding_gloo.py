"""Tree sharding across ranks (the reference's multi-GPU scheme: GpuAlgorithm
splits the trees over devices, gpu_algorithm.cc:17-50, and sums the votes,
ml_resultdata_impl.cc:62-71) with world_size 2 over gloo on CPU: each rank
fits its share of the trees with tree_offset = the trees before it, the vote
arrays are all-reduced, and the sum equals the single forest's votes.  The
oracle stands in for the engine (no GPU here); the engine's own parts-equal-
whole property is tested on the GPU (test_tree_offset_parts_equal_the_whole_forest)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _shard(n_trees, world, rank):
    per, extra = divmod(n_trees, world)
    first = rank * per + min(rank, extra)
    return first, per + (1 if rank < extra else 0)


def _worker(rank, world, port, kw, out_path):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    sys.path.insert(0, os.path.dirname(HERE))
    import oracle
    from datamininglibs_gb300 import synth
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    X, y = synth.rf_multiclass(1500, 12, n_classes=3, n_int=2, seed=4)
    first, count = _shard(kw["n_trees"], world, rank)
    part = dict(kw, n_trees=count)
    m = oracle.fit(X, y, tree_offset=first, threads=1, **part)
    votes = torch.from_numpy(oracle.predict(m, X, threads=1))
    dist.all_reduce(votes, op=dist.ReduceOp.SUM)
    # the bench's timing rule: the slowest rank's time is the job's time
    t = torch.tensor([float(rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        np.save(out_path, votes.numpy())
        assert t.item() == float(world)
    dist.destroy_process_group()


@pytest.mark.parametrize("n_trees", [6, 7])
def test_tree_shards_over_two_ranks_sum_to_the_whole_forest(tmp_path, n_trees):
    import oracle
    from datamininglibs_gb300 import synth
    kw = dict(algo=0, n_trees=n_trees, K=4, max_depth=10, min_node_size=5, n_classes=3, seed=9)
    out = str(tmp_path / "votes.npy")
    mp.start_processes(_worker, args=(2, _free_port(), kw, out), nprocs=2, join=True,
                       start_method="spawn")
    X, y = synth.rf_multiclass(1500, 12, n_classes=3, n_int=2, seed=4)
    whole = oracle.predict(oracle.fit(X, y, threads=1, **kw), X, threads=1)
    assert np.array_equal(np.load(out), whole)
