"""Many independent circuits of different sizes: forward + adjoint gradients.

Circuits are grouped by structure (modes, cutoff, gate list); each group is
one batched ``CompiledCircuit`` whose kernels index the circuit with
``blockIdx.z`` (parameters per circuit, one gate structure).  Groups run on a
small pool of CUDA streams so small groups overlap, and large circuits keep
only every ``checkpoint``-th state for the adjoint sweep.  This replaces the
reference's one-circuit-at-a-time engine loop (``LocalEngine._run_program``,
strawberryfields/engine.py:422-471) and generalises the TF backend's
same-shape batch axis (``tfbackend/circuit.py:129-185``) to heterogeneous
circuits.
"""

import numpy as np
import torch

from .autograd import CompiledCircuit


def fidelity_loss_grad(psi, target):
    """L = 1 - |<t|psi>|^2 per circuit of a batch and dL/dpsi (torch
    convention dL/dRe + i dL/dIm), summed over nothing (one value per circuit)."""
    dims = tuple(range(1, psi.dim()))
    s = torch.sum(target.conj() * psi, dim=dims)
    loss = 1 - (s.real ** 2 + s.imag ** 2)
    g = -2 * s.reshape((-1,) + (1,) * (psi.dim() - 1)) * target
    return loss, g


class CircuitBatch:
    """Independent circuits run as structure groups.

    Args:
        circuits (Sequence[tuple]): ``(num_modes, cutoff, gates, n_params)``
            per circuit (``gates`` as for :class:`CompiledCircuit`)
        dtype: state precision (default complex64)
        device: CUDA device
        streams (int): CUDA streams the groups are spread over
        checkpoint_bytes (int): groups whose stored states would exceed this
            many bytes keep only checkpoints (every k-th state)
    """

    def __init__(self, circuits, dtype=torch.complex64, device=None, streams=8, checkpoint_bytes=8 << 30):
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.dtype = dtype
        self.n = len(circuits)
        groups = {}
        for i, (nm, D, gates, npar) in enumerate(circuits):
            key = (int(nm), int(D), tuple(tuple(int(v) for v in g) for g in gates), int(npar))
            groups.setdefault(key, []).append(i)
        esz = 8 if dtype == torch.complex64 else 16
        self.groups = []
        # largest work first so the long groups start early
        order = sorted(groups.items(), key=lambda kv: -(kv[0][1] ** kv[0][0]) * len(kv[0][2]) * len(kv[1]))
        for key, idx in order:
            nm, D, gates, npar = key
            probe = CompiledCircuit(nm, D, list(gates), npar, dtype=dtype, device=self.device, batch=1)
            n_ops = probe.n_ops
            del probe
            stored = n_ops * len(idx) * (D ** nm) * esz
            k = 1
            if stored > checkpoint_bytes:
                k = max(2, int(np.ceil(np.sqrt(n_ops))))
            circ = CompiledCircuit(nm, D, list(gates), npar, dtype=dtype, device=self.device, batch=len(idx),
                                   checkpoint=k)
            self.groups.append({"key": key, "idx": np.array(idx), "circ": circ, "n_ops": n_ops})
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(max(1, streams))]

    def stats(self):
        """Groups, fused ops and algorithmic bytes of one forward + adjoint."""
        esz = 8 if self.dtype == torch.complex64 else 16
        fwd = bwd = 0
        for g in self.groups:
            nm, D = g["key"][0], g["key"][1]
            S = (D ** nm) * esz * len(g["idx"])
            fwd += 2 * S * g["n_ops"]
            bwd += 3 * S * g["n_ops"]
        return {"circuits": self.n, "groups": len(self.groups),
                "ops": int(sum(g["n_ops"] * len(g["idx"]) for g in self.groups)),
                "bytes_forward": fwd, "bytes_adjoint": bwd}

    def value_and_grad(self, params, targets):
        """Loss and gradient of every circuit.

        Args:
            params (Sequence[torch.Tensor]): per-circuit float64 parameter
                vectors on the device
            targets (dict): (num_modes, cutoff) -> target ket tensor
        Returns:
            (losses, grads): lists indexed like the circuits
        """
        losses = [None] * self.n
        grads = [None] * self.n
        cur = torch.cuda.current_stream(self.device)
        for gi, g in enumerate(self.groups):
            st = self.streams[gi % len(self.streams)]
            st.wait_stream(cur)
            with torch.cuda.stream(st):
                circ = g["circ"]
                idx = g["idx"]
                p = torch.stack([params[i] for i in idx]) if len(idx) > 1 else params[idx[0]]
                states = circ.forward_states(p)
                psi = states[circ.final_index()]
                t = targets[(g["key"][0], g["key"][1])].to(circ.dtype)
                if len(idx) > 1:
                    loss, gpsi = fidelity_loss_grad(psi, t.unsqueeze(0).expand_as(psi))
                else:
                    loss, gpsi = fidelity_loss_grad(psi.unsqueeze(0), t.unsqueeze(0))
                    gpsi = gpsi[0]
                gr, _ = circ.backward(p, states, gpsi)
                del states
                circ.release()
                if len(idx) > 1:
                    for j, i in enumerate(idx):
                        losses[i] = loss[j]
                        grads[i] = gr[j]
                else:
                    losses[idx[0]] = loss[0]
                    grads[idx[0]] = gr
        for st in self.streams:
            cur.wait_stream(st)
        return losses, grads


def random_qnn_batch(n_circuits, seed=0, modes=(2, 5), cutoffs=(6, 20), depths=(2, 10)):
    """The heterogeneous CV-QNN workload: modes, cutoff and depth uniform in
    the given inclusive ranges, parameters seeded per circuit."""
    from .qnn import qnn_gates, qnn_params

    rng = np.random.default_rng(seed)
    circuits, params = [], []
    for i in range(n_circuits):
        nm = int(rng.integers(modes[0], modes[1] + 1))
        D = int(rng.integers(cutoffs[0], cutoffs[1] + 1))
        depth = int(rng.integers(depths[0], depths[1] + 1))
        gates, npar = qnn_gates(nm, depth)
        circuits.append((nm, D, gates, npar))
        params.append(qnn_params(gates, npar, seed=seed * 1_000_003 + i))
    return circuits, params
