"""Batched circuits across ranks: cost-balanced sharding and the one gather (gloo, 2 ranks, CPU).

Each rank evaluates its share with a CPU runner (the oracle plus numpy energies), standing in
for the GPU runner; the test checks that every circuit lands exactly once and every rank ends
with the same energies and gradient slots as a single-process run (one all-reduce of flat arrays).
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from quantr_gb300 import batch as B  # noqa: E402
from quantr_gb300 import workloads as W  # noqa: E402


def _circuits():
    return B.batch_config(count=12, seed=9, layers=2, n_min=3, n_max=6)


def _cpu_runner(cs):
    from oracle import oracle as orc

    es = [W.energy_dense(orc.simulate(c.program, engine=orc.DENSE), c.a, c.b) for c in cs]
    # stand-in gradients that identify their circuit, so the gather of the gradient slots is checked
    return np.array(es), [e + np.arange(len(c.program.ops)) * 1e-3 for e, c in zip(es, cs)]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        e, g = B.run_distributed(_circuits(), runner=_cpu_runner)
        np.save(os.path.join(out_dir, f"e{rank}.npy"), e)
        np.save(os.path.join(out_dir, f"g{rank}.npy"), np.concatenate(g))
    finally:
        dist.destroy_process_group()


def test_shard_balances_and_covers():
    cs = _circuits()
    parts = B.shard(cs, 3)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(cs)))
    loads = [sum(cs[i].cost() for i in p) for p in parts]
    assert max(loads) <= 2.0 * (sum(loads) / 3) + max(c.cost() for c in cs)


def test_two_rank_gather_matches_single_process(tmp_path):
    ref, refg = _cpu_runner(_circuits())
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        e = np.load(tmp_path / f"e{r}.npy")
        assert np.allclose(e, ref, atol=1e-12, rtol=0)
        assert np.allclose(np.load(tmp_path / f"g{r}.npy"), np.concatenate(refg), atol=1e-12, rtol=0)


def test_shard_meets_the_list_scheduling_bound():
    """Largest-first greedy sharding of uneven batches (10..24 qubits, as the batching
    configuration draws them) over 1..8 ranks: every circuit exactly once, the heaviest rank at
    most the average load plus one circuit, and no rank idle while circuits outnumber ranks."""
    class _C:
        def __init__(self, c):
            self.c = c

        def cost(self):
            return self.c

    rng = np.random.default_rng(4)
    for trial in range(40):
        count = int(rng.integers(1, 300))
        cs = [_C(float(2 ** int(rng.integers(10, 25)) * int(rng.integers(20, 200))))
              for _ in range(count)]
        for world in range(1, 9):
            parts = B.shard(cs, world)
            assert len(parts) == world
            assert sorted(i for p in parts for i in p) == list(range(count))
            loads = [sum(cs[i].cost() for i in p) for p in parts]
            assert max(loads) <= sum(loads) / world + max(c.cost() for c in cs)
            if count >= world:
                assert min(len(p) for p in parts) >= 1
