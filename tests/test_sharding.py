"""Circuit-queue sharding across ranks (strawberryfields_gb300/sharding.py):
the cost partition, and the gathered per-circuit results of a gloo world of
two ranks on CPU against one rank doing everything.  The ranks' local runner
here is the oracle (CPU); on GPUs it is a CircuitBatch per rank."""
import os
import socket

import numpy as np
import pytest

from oracle import fock_oracle as fo


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


class OracleRunner:
    """Loss 1 - |<t|psi>|^2 and its gradient per circuit, on the CPU oracle."""

    def __init__(self, circuits):
        self.circuits = circuits

    def value_and_grad(self, params, targets):
        losses, grads = [], []
        for (nm, D, gates, _), p in zip(self.circuits, params):
            t = targets[(nm, D)]
            psi = fo.run_gates(gates, p, nm, D)[-1]
            s = np.vdot(t, psi)
            losses.append(1 - abs(s) ** 2)
            grads.append(fo.adjoint_grads(gates, p, nm, D, -2 * s * t))
        return losses, grads


def _workload():
    from strawberryfields_gb300.batch import random_qnn_batch
    from strawberryfields_gb300.qnn import target_state

    circuits, params = random_qnn_batch(12, seed=5, modes=(2, 3), cutoffs=(3, 6), depths=(1, 3))
    targets = {(nm, D): target_state(nm, D, 2, seed=nm * 100 + D) for nm, D, _, _ in circuits}
    return circuits, params, targets


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from strawberryfields_gb300.sharding import ShardedBatch

    circuits, params, targets = _workload()
    sb = ShardedBatch(circuits, rank, world, runner=OracleRunner)
    losses, grads = sb.value_and_grad(params, targets)
    out[rank] = (sb.mine, [float(x) for x in losses], [np.asarray(g).tolist() for g in grads])
    dist.destroy_process_group()


def test_partition_covers_every_circuit_once_and_balances():
    from strawberryfields_gb300.sharding import partition_by_cost

    rng = np.random.default_rng(0)
    costs = rng.pareto(1.5, size=500) + 1.0
    for world in (1, 2, 3, 8):
        shares, loads = partition_by_cost(costs, world)
        flat = sorted(i for s in shares for i in s)
        assert flat == list(range(len(costs)))
        assert np.allclose(loads, [costs[s].sum() for s in shares])
        # greedy longest-first: the largest load exceeds the mean by at most
        # one circuit's cost
        assert loads.max() <= costs.sum() / world + costs.max() + 1e-9


def test_partition_of_the_4096_circuit_workload():
    """The heterogeneous CV-QNN workload (modes U{2..5}, cutoff U{6..20},
    depth U{2..10}, seed 0) over 2 and 8 ranks: rank loads within 1% of the
    mean."""
    from strawberryfields_gb300.batch import random_qnn_batch
    from strawberryfields_gb300.sharding import circuit_cost, partition_by_cost

    circuits, _ = random_qnn_batch(4096, seed=0)
    costs = np.array([circuit_cost(nm, D, g) for nm, D, g, _ in circuits])
    for world in (2, 8):
        shares, loads = partition_by_cost(costs, world)
        assert sum(len(s) for s in shares) == 4096
        assert loads.max() / loads.mean() < 1.01


def test_sharded_results_equal_single_rank():
    import torch.multiprocessing as mp

    from strawberryfields_gb300.sharding import ShardedBatch

    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    circuits, params, targets = _workload()
    ref_l, ref_g = ShardedBatch(circuits, 0, 1, runner=OracleRunner).value_and_grad(params, targets)
    mine0, mine1 = out[0][0], out[1][0]
    assert sorted(mine0 + mine1) == list(range(len(circuits)))
    assert not set(mine0) & set(mine1)
    assert mine0 and mine1
    for r in range(2):
        _, losses, grads = out[r]
        assert losses == [float(x) for x in ref_l]
        for g, rg in zip(grads, ref_g):
            assert np.array_equal(np.asarray(g), np.asarray(rg))
