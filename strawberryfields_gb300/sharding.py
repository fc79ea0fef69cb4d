"""Independent circuits sharded across ranks (one GPU per rank).

A queue of heterogeneous circuits (different modes, cutoffs and depths) has no
data dependence between circuits, so it partitions with no collective on the
data path: every rank simulates its share on its own GPU and the per-circuit
losses and gradients are gathered on the host afterwards.  Shares are balanced
by the circuits' algorithmic cost -- state bytes times non-diagonal gate
passes, S * G_nd, the bytes one forward sweep moves per pass -- with the
longest-processing-time-first rule: circuits in decreasing cost, each to the
least-loaded rank.  That rule keeps the largest rank load within
(4/3 - 1/(3 m)) of the best possible for m ranks (Graham 1969), and within one
circuit's cost of the mean load.

The reference runs one circuit at a time in one process
(``LocalEngine._run_program``, strawberryfields/engine.py:422-471); it has no
multi-device path.
"""

import numpy as np

from . import _lib as L

_DIAGONAL = (L.ROTATION, L.KERR, L.CROSS_KERR)


def circuit_cost(num_modes, cutoff, gates, pure=True, elem_bytes=8):
    """S * G_nd of one circuit: state bytes times the gates that are not
    diagonal (rotations, Kerr and cross-Kerr are fused into other passes)."""
    g_nd = sum(1 for g in gates if int(g[0]) not in _DIAGONAL)
    naxes = num_modes if pure else 2 * num_modes
    return float(cutoff) ** naxes * elem_bytes * max(g_nd, 1)


def partition_by_cost(costs, world):
    """Longest processing time first: returns (shares, loads) with
    ``shares[r]`` the sorted circuit indices of rank r.  Deterministic (ties
    by circuit index, then by rank)."""
    if world < 1:
        raise ValueError("world size must be positive")
    costs = np.asarray(costs, dtype=np.float64)
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    loads = np.zeros(world)
    shares = [[] for _ in range(world)]
    for i in order:
        r = int(np.argmin(loads))  # first least-loaded rank
        shares[r].append(i)
        loads[r] += costs[i]
    return [sorted(s) for s in shares], loads


class ShardedBatch:
    """A circuit queue split across the ranks of a ``torch.distributed``
    process group; each rank runs its share with ``runner`` and the results
    are gathered on the host.

    Args:
        circuits (Sequence[tuple]): ``(num_modes, cutoff, gates, n_params)``
            per circuit (as for :class:`~strawberryfields_gb300.batch.CircuitBatch`)
        rank, world (int): this process's rank and the group size
        runner (callable): builds the local runner from this rank's circuits
            (default: a :class:`~strawberryfields_gb300.batch.CircuitBatch` on
            the current GPU); the runner's ``value_and_grad(params, targets)``
            returns per-circuit losses and gradients
        group: process group for the gather (default: the world group)
    """

    def __init__(self, circuits, rank, world, runner=None, group=None, **runner_kwargs):
        self.circuits = list(circuits)
        self.rank, self.world, self.group = int(rank), int(world), group
        costs = [circuit_cost(nm, D, gates) for nm, D, gates, _ in self.circuits]
        self.shares, self.loads = partition_by_cost(costs, self.world)
        self.mine = self.shares[self.rank]
        if runner is None:
            from .batch import CircuitBatch

            runner = CircuitBatch
        local = [self.circuits[i] for i in self.mine]
        self.local = runner(local, **runner_kwargs) if local else None

    def value_and_grad(self, params, targets):
        """Every circuit's loss and gradient, on every rank, ordered like the
        circuits: this rank computes its share, then one host gather (no
        device collective)."""
        import torch
        import torch.distributed as dist

        mine = {}
        if self.local is not None:
            losses, grads = self.local.value_and_grad([params[i] for i in self.mine], targets)
            for j, i in enumerate(self.mine):
                mine[i] = (float(torch.as_tensor(losses[j]).reshape(())),
                           torch.as_tensor(grads[j]).detach().reshape(-1).cpu().numpy())
        if self.world > 1 and dist.is_available() and dist.is_initialized():
            gathered = [None] * self.world
            dist.all_gather_object(gathered, mine, group=self.group)
        else:
            gathered = [mine]
        out_l, out_g = [None] * len(self.circuits), [None] * len(self.circuits)
        for part in gathered:
            for i, (l, g) in part.items():
                out_l[i], out_g[i] = l, g
        return out_l, out_g
