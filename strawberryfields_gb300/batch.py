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
        # flat parameter layout: circuit order, and the same entries group by group
        npar = [int(c[3]) for c in circuits]
        self.param_offsets = np.concatenate([[0], np.cumsum(npar)]).astype(np.int64)
        order = []
        for g in self.groups:
            for i in g["idx"]:
                order.extend(range(self.param_offsets[i], self.param_offsets[i + 1]))
        self._gather = torch.as_tensor(np.array(order, dtype=np.int64), device=self.device)
        # circuit index of every loss in group order
        self._order = torch.as_tensor(np.concatenate([g["idx"] for g in self.groups]).astype(np.int64),
                                      device=self.device)
        self.graph = None

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


    def _group_params(self, flat_group):
        """Per-group parameter views ([batch, n_params]) of a group-ordered
        flat vector."""
        out, o = [], 0
        for g in self.groups:
            nb, npar = len(g["idx"]), g["key"][3]
            out.append(flat_group[o:o + nb * npar].view(nb, npar) if nb > 1 else flat_group[o:o + npar])
            o += nb * npar
        return out

    def _step(self, flat_params, targets, losses, grads):
        """One step on group-ordered views: every group's forward, loss and
        adjoint, results scattered into losses [n] and grads (flat, circuit
        order)."""
        flat_group = flat_params.index_select(0, self._gather)
        gparams = self._group_params(flat_group)
        cur = torch.cuda.current_stream(self.device)
        gl, gg = [], []
        for gi, g in enumerate(self.groups):
            st = self.streams[gi % len(self.streams)]
            st.wait_stream(cur)
            with torch.cuda.stream(st):
                circ, idx = g["circ"], g["idx"]
                p = gparams[gi]
                states = circ.forward_states(p)
                psi = states[circ.final_index()]
                t = targets[(g["key"][0], g["key"][1])].to(circ.dtype)
                if len(idx) > 1:
                    loss, gpsi = fidelity_loss_grad(psi, t.unsqueeze(0).expand_as(psi))
                else:
                    loss, gpsi = fidelity_loss_grad(psi.unsqueeze(0), t.unsqueeze(0))
                    gpsi = gpsi[0]
                gr, _ = circ.backward(p, states, gpsi)
                del states, psi, gpsi
                circ.release()
                gl.append(loss.reshape(-1))
                gg.append(gr.reshape(-1))
        for st in self.streams:
            cur.wait_stream(st)
        losses.index_copy_(0, self._order, torch.cat(gl).to(losses.dtype))
        grads.index_copy_(0, self._gather, torch.cat(gg))

    def capture(self, params, targets, warmup=1):
        """Capture one whole step -- every group's forward sweep, loss and
        adjoint sweep on the group streams -- as a single CUDA graph.  Returns
        ``step(flat_params=None) -> (losses [n], grads flat)``; parameters are
        a flat circuit-order vector (``param_offsets`` per circuit) copied into
        the graph's input buffer before each replay."""
        flat = torch.cat([torch.as_tensor(p, device=self.device, dtype=torch.float64).reshape(-1) for p in params])
        self._in = flat.clone()
        self._losses = torch.zeros(self.n, dtype=torch.float64, device=self.device)
        self._grads = torch.zeros_like(flat)
        cur = torch.cuda.current_stream(self.device)
        side = torch.cuda.Stream(device=self.device)
        side.wait_stream(cur)
        with torch.cuda.stream(side):
            for _ in range(warmup):
                self._step(self._in, targets, self._losses, self._grads)
        cur.wait_stream(side)
        torch.cuda.synchronize(self.device)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._step(self._in, targets, self._losses, self._grads)

        def step(flat_params=None):
            if flat_params is not None:
                self._in.copy_(flat_params, non_blocking=True)
            self.graph.replay()
            return self._losses, self._grads

        return step


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
