"""Differentiable compiled circuits: forward sweep + adjoint sweep on the GPU.

``CompiledCircuit`` compiles a gate list once (``fock_plan_create``: diagonal
gates fused into their neighbours) and runs it as a function of a device
parameter vector.  Calling it goes through a ``torch.autograd.Function`` whose
backward is the hand-written adjoint sweep (``fock_plan_backward``): the
reverse pass applies M^dagger to the adjoint state and contracts it with the
stored forward states, then maps dL/dM to dL/dparams through the FP64 gate
derivatives -- the gradient contract of the reference's TF backend
(``strawberryfields/backends/tfbackend/ops.py:190-454`` custom gradients and
the einsum applies at :688-854), without a tape.

This path also bypasses ``Program.compile`` and the per-gate host loop of
``LocalEngine._run_program`` (engine.py:422-471), which dominate small
circuits in the reference.
"""

import ctypes

import torch

from . import _lib as L
from .circuit import _dtype_code


class CompiledCircuit:
    """A gate list compiled for the GPU.

    Args:
        num_modes (int): number of modes
        cutoff (int): Fock cutoff D
        gates (Sequence[tuple]): ``(kind, mode1, mode2, pidx)`` per gate, kinds
            from :mod:`strawberryfields_gb300._lib` (``mode2 = -1`` for
            single-mode gates); gate parameters are ``params[pidx]`` and
            ``params[pidx + 1]``
        n_params (int): length of the parameter vector
        dtype: ``torch.complex64`` (default) or ``torch.complex128`` state
        device: CUDA device
        batch (int): number of circuits of this structure run together, each
            with its own parameters (parameters ``[batch, n_params]``, states
            ``[batch, D, ..., D]``) -- the batch axis of the reference's TF
            backend (``tfbackend/circuit.py:129-185``); 1 gives unbatched shapes
        checkpoint (int): keep every ``checkpoint``-th op output for the
            adjoint sweep and recompute the others segment by segment (1 keeps
            all outputs; larger values trade one extra forward for
            ``n_ops / checkpoint + checkpoint`` resident states instead of ``n_ops``)
        pure (bool): ket ``[D]*n`` (default) or density matrix ``[D]*(2n)``
            with interleaved (ket, bra) axes; mixed circuits may contain
            ``LOSS`` gates (parameter T)
        recompute_slots (int): states the backward sweep may hold while it
            recomputes a checkpoint segment (default ``checkpoint - 1``: the
            whole segment); fewer (at least 3) recompute the segment
            recursively in bounded memory
    """

    def __init__(self, num_modes, cutoff, gates, n_params, dtype=torch.complex64, device=None, batch=1,
                 checkpoint=1, pure=True, recompute_slots=None):
        lib = L.load()
        self.num_modes = int(num_modes)
        self.cutoff = int(cutoff)
        self.n_params = int(n_params)
        self._dcode, self.dtype = _dtype_code(dtype)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        arr = (L.FockGate * max(len(gates), 1))()
        for i, g in enumerate(gates):
            kind, m1, m2, pidx = g
            arr[i].kind, arr[i].mode1, arr[i].mode2, arr[i].pidx = int(kind), int(m1), int(m2), int(pidx)
        plan = ctypes.c_void_p()
        self.batch = int(batch)
        self.checkpoint = int(checkpoint)
        self.pure = bool(pure)
        if self.checkpoint < 1:
            raise ValueError("checkpoint must be >= 1")
        self.recompute_slots = max(self.checkpoint - 1, 1) if recompute_slots is None else int(recompute_slots)
        L.check(lib.fock_plan_create_batch(self.num_modes, self.cutoff, 1 if self.pure else 0, self._dcode, arr,
                                           len(gates), self.n_params, self.batch, ctypes.byref(plan)),
                "fock_plan_create")
        self._plan = plan
        info = L.PlanInfo()
        L.check(lib.fock_plan_get_info(plan, ctypes.byref(info)), "fock_plan_get_info")
        self.info = info
        self.n_gates = len(gates)
        self.shape = [self.cutoff] * (self.num_modes if self.pure else 2 * self.num_modes)
        self._bshape = ([self.batch] if self.batch > 1 else []) + self.shape
        self._ws_buf = None
        # the workspace's matrices were built by forward sweep number _fwd_n
        # for the parameter buffer (data pointer, version) _built_for
        self._fwd_n = 0
        self._built_for = None
        self._vacuum = torch.zeros([self.batch, int(info.state_elems)], dtype=self.dtype, device=self.device)
        self._vacuum[:, 0] = 1.0
        self._vacuum = self._vacuum.reshape(self._bshape)

    def __del__(self):
        plan = getattr(self, "_plan", None)
        if plan is not None and plan.value:
            try:
                L.load().fock_plan_destroy(plan)
            except Exception:  # interpreter shutdown
                pass
            self._plan = None

    @property
    def _ws(self):
        """Workspace (allocated on first use; ``release()`` returns it)."""
        if self._ws_buf is None:
            self._ws_buf = torch.empty(int(self.info.workspace_bytes), dtype=torch.uint8, device=self.device)
        return self._ws_buf

    def release(self):
        """Drop the workspace until the next sweep (memory reuse across plans)."""
        self._ws_buf = None
        self._built_for = None

    @property
    def n_ops(self):
        return int(self.info.n_ops)

    def ops(self):
        """Fused ops: list of (kind, mode1, mode2, n_gates_fused)."""
        lib = L.load()
        out = []
        for k in range(self.n_ops):
            a, b, c, d = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
            L.check(lib.fock_plan_op(self._plan, k, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                     ctypes.byref(d)))
            out.append((a.value, b.value, c.value, d.value))
        return out

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def _params(self, params):
        p = torch.as_tensor(params)
        if p.device != self.device or p.dtype != torch.float64:
            p = p.to(device=self.device, dtype=torch.float64)
        if p.numel() != self.n_params * self.batch:
            raise ValueError(f"expected {self.batch} x {self.n_params} parameters, got {tuple(p.shape)}")
        return p.contiguous()

    def _slots(self, k):
        n = self.n_ops
        if k <= 0:
            return 2
        if k == 1:
            return n
        return -(-n // k) + 2

    def final_index(self, k=None):
        """Slot of the final state in a forward sweep with store_every = k."""
        k = self.checkpoint if k is None else k
        n = self.n_ops
        if k <= 0:
            return (n - 1) & 1
        if k == 1:
            return n - 1
        return -(-n // k) - 1

    def forward_states(self, params, state_in=None, store_all=True, store_every=None):
        """Run the forward sweep and return the kept states ([slots, ...]):
        every op output (``store_every=1``), checkpoints (``> 1``), or, with
        ``store_all=False``, only the final state."""
        p = self._params(params)
        x = self._vacuum if state_in is None else state_in.to(self.dtype).contiguous()
        n = self.n_ops
        if n == 0:
            return x.clone().unsqueeze(0)
        k = (self.checkpoint if store_every is None else int(store_every)) if store_all else 0
        states = torch.empty([self._slots(k)] + self._bshape, dtype=self.dtype, device=self.device)
        L.check(L.load().fock_plan_forward(self._plan, p.data_ptr(), x.data_ptr(), states.data_ptr(),
                                           k, self._ws.data_ptr(), self._stream()),
                "fock_plan_forward")
        self._fwd_n += 1
        self._built_for = (p.data_ptr(), p._version, self._fwd_n)
        if not store_all:
            return states[self.final_index(0)]
        return states

    def backward(self, params, states, grad_state, state_in=None, overwrite_grad=False):
        """Adjoint sweep: returns (dL/dparams, dL/dstate_in) given dL/dpsi_final.
        With ``overwrite_grad`` a contiguous ``grad_state`` of the state dtype
        is used as the sweep's buffer (and holds dL/dstate_in afterwards)
        instead of a copy."""
        p = self._params(params)
        x = self._vacuum if state_in is None else state_in.to(self.dtype).contiguous()
        if overwrite_grad and grad_state.dtype == self.dtype and grad_state.is_contiguous():
            lam = grad_state
        else:
            lam = grad_state.to(self.dtype).contiguous().clone()
        tmp = torch.empty_like(lam)
        grads = torch.empty(([self.batch] if self.batch > 1 else []) + [self.n_params], dtype=torch.float64,
                            device=self.device)
        if self.n_ops == 0:
            grads.zero_()
            return grads, lam
        k = self.checkpoint
        nslot = self.recompute_slots
        seg = torch.empty([nslot] + self._bshape, dtype=self.dtype, device=self.device) if k > 1 else None
        # the last forward sweep on this workspace built the matrices for the
        # same parameter buffer, unmodified since: skip the rebuild
        reuse = self._ws_buf is not None and self._built_for == (p.data_ptr(), p._version, self._fwd_n)
        flags = L.FOCK_BACKWARD_REUSE_BUILD if reuse else 0
        L.check(L.load().fock_plan_backward_recompute(self._plan, p.data_ptr(), x.data_ptr(), states.data_ptr(), k,
                                                      seg.data_ptr() if seg is not None else None, nslot,
                                                      lam.data_ptr(), tmp.data_ptr(), grads.data_ptr(), flags,
                                                      self._ws.data_ptr(), self._stream()),
                "fock_plan_backward_recompute")
        return grads, lam

    def op_config(self, k):
        """(family, adjoint CTAs per SM, plane_ok, plane tile columns) of
        fused op k: family 0 is the block kernels, 1 the plane-tile kernels."""
        fam, ctas, ok, tc = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        L.check(L.load().fock_plan_op_config(self._plan, int(k), ctypes.byref(fam), ctypes.byref(ctas),
                                             ctypes.byref(ok), ctypes.byref(tc)), "fock_plan_op_config")
        return fam.value, ctas.value, bool(ok.value), tc.value

    def tune_op(self, k, family=-1, ctas_per_sm=0, tile_columns=0):
        """Select op k's kernel family (-1 keeps it), block-adjoint CTAs per
        SM and plane tile columns of a two-mode op (0 keeps them).
        Reallocates the workspace on the next sweep; graphs captured before
        the change are stale."""
        torch.cuda.synchronize(self.device)
        L.check(L.load().fock_plan_tune(self._plan, int(k), int(family), int(ctas_per_sm), int(tile_columns)),
                "fock_plan_tune")
        info = L.PlanInfo()
        L.check(L.load().fock_plan_get_info(self._plan, ctypes.byref(info)), "fock_plan_get_info")
        self.info = info
        self.release()

    def _timed_sweeps(self, p, lam, repeats, per_op):
        """Best-of-``repeats`` device times of one forward + adjoint sweep:
        per op (fwd_ms, bwd_ms) arrays with ``per_op``, else the whole step in ms."""
        lib = L.load()
        n = self.n_ops
        fbuf, bbuf = (ctypes.c_float * n)(), (ctypes.c_float * n)()
        best_f, best_b, best = [float("inf")] * n, [float("inf")] * n, float("inf")
        st = torch.cuda.current_stream(self.device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for r in range(repeats + 1):  # the first sweep warms up
            e0.record(st)
            states = self.forward_states(p)
            self.backward(p, states, lam)
            e1.record(st)
            torch.cuda.synchronize(self.device)
            if r == 0:
                continue
            best = min(best, e0.elapsed_time(e1))
            if per_op:
                L.check(lib.fock_plan_op_times(self._plan, fbuf, bbuf), "fock_plan_op_times")
                best_f = [min(a, b) for a, b in zip(best_f, fbuf)]
                best_b = [min(a, b) for a, b in zip(best_b, bbuf)]
        return (best_f, best_b) if per_op else best

    def autotune(self, params, ctas=(2, 4, 6, 8, 12, 16), tiles=(32, 24, 16), repeats=3):
        """Pick each op's kernel family, block-adjoint CTAs per SM and plane
        tile columns by timing a forward + adjoint sweep at ``params`` under
        every candidate (per-op CUDA events, best of ``repeats``), keeping per
        op the candidate with the smallest forward + adjoint time.  The whole
        step (PDL launches, final reduction) then decides between these picks,
        the picks with the starting CTA densities, each with one plane tile
        width for every plane op, and the configuration it started from.  Returns
        ``(configs, ms_before, ms_after)`` with configs[k] =
        (family, ctas, tile columns)."""
        if self.n_ops == 0:
            return [], 0.0, 0.0
        lib = L.load()
        p = self._params(params)
        g = torch.Generator(device="cpu").manual_seed(0)
        lam = torch.complex(torch.randn(self._bshape, generator=g, dtype=torch.float64),
                            torch.randn(self._bshape, generator=g, dtype=torch.float64))
        lam = (lam / lam.abs().pow(2).sum().sqrt()).to(device=self.device, dtype=self.dtype)
        n = self.n_ops
        start = [self.op_config(k) for k in range(n)]
        ms_before = self._timed_sweeps(p, lam, repeats, False)
        cands = [(0, int(c), 0) for c in ctas]
        if any(ok for _, _, ok, _ in start):
            cands += [(1, 0, int(t)) for t in tiles]
        cost = [dict() for _ in range(n)]
        L.check(lib.fock_plan_enable_timing(self._plan, 1), "fock_plan_enable_timing")
        try:
            for fam, c, tc in cands:
                for k in range(n):
                    if fam == 0 or start[k][2]:
                        self.tune_op(k, fam, c, tc if start[k][3] <= 32 else 0)
                    else:
                        self.tune_op(k, 0, start[k][1])
                f, b = self._timed_sweeps(p, lam, repeats, True)
                for k in range(n):
                    if fam == 0 or start[k][2]:
                        cost[k][(fam, c, tc)] = f[k] + b[k]
        finally:
            L.check(lib.fock_plan_enable_timing(self._plan, 0), "fock_plan_enable_timing")
        best = [min(ck, key=ck.get) for ck in cost]

        def tile(k, tc):
            return tc if start[k][3] <= 32 else 0

        def apply(cfg):
            for k, (fam, c, tc) in enumerate(cfg):
                self.tune_op(k, fam, c, tile(k, tc))

        # whole-step check of the per-op picks, of the picks with the
        # starting CTA densities (per-op events run without programmatic
        # dependent launch, which favours other densities), and of the start
        start_cfg = [(fam, c, tc) for fam, c, _, tc in start]
        # (an op left on block kernels keeps its starting plane tile)
        picks = [(fam, c if fam == 0 else start[k][1], tc if fam == 1 else start[k][3])
                 for k, (fam, c, tc) in enumerate(best)]
        no_ctas = [(fam, start[k][1], tc) for k, (fam, c, tc) in enumerate(picks)]
        # and of one tile width for every plane op: per-op events favour wider
        # tiles on the adjoint, while the step on an L2-resident state can
        # prefer the narrower tiles' extra resident CTAs for every plane op
        uniform = [[(fam, c, tw if fam == 1 else tc) for fam, c, tc in base]
                   for tw in tiles for base in (picks, no_ctas) if any(f == 1 for f, _, _ in base)]
        results = [(ms_before, start_cfg)]
        for cfg in [picks, no_ctas] + uniform:
            if cfg != start_cfg and all(cfg != r[1] for r in results):
                apply(cfg)
                results.append((self._timed_sweeps(p, lam, repeats, False), cfg))
        ms_after, cfg = min(results, key=lambda r: r[0])
        apply(cfg)
        self.tuned = [(fam, c, tc) for fam, c, _, tc in (self.op_config(k) for k in range(n))]
        return self.tuned, ms_before, ms_after

    def sweep_status(self):
        """(persistent, error): whether this plan runs its sweeps as single
        persistent launches, and whether a grid barrier of the last such sweep
        gave up (outputs invalid).  Synchronises the device."""
        torch.cuda.synchronize(self.device)
        grids, err = (ctypes.c_int * 2)(), ctypes.c_int()
        ws = self._ws_buf.data_ptr() if self._ws_buf is not None else None
        L.check(L.load().fock_plan_sweep_status(self._plan, ws, grids, ctypes.byref(err) if ws else None),
                "fock_plan_sweep_status")
        self.sweep_grids = (grids[0], grids[1])
        return grids[0] > 0, int(err.value)

    def __call__(self, params, state_in=None):
        """Final state as a differentiable function of ``params``."""
        return _CircuitFunction.apply(params, self, state_in)


class _CircuitFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, circ, state_in):
        states = circ.forward_states(params.detach(), state_in)
        ctx.circ = circ
        ctx.state_in = state_in
        ctx.save_for_backward(params.detach(), states)
        return states[circ.final_index()].clone() if circ.n_ops else states[0]

    @staticmethod
    def backward(ctx, grad_out):
        params, states = ctx.saved_tensors
        grads, lam = ctx.circ.backward(params, states, grad_out, ctx.state_in)
        gin = lam if (ctx.state_in is not None and ctx.needs_input_grad[2]) else None
        return grads.to(params.dtype), None, gin


class GraphedGradient:
    """One gradient step -- fused forward sweep, the loss, the adjoint sweep --
    captured once as a CUDA graph and replayed (the spec design: the
    whole forward+backward as one graph launch, no per-kernel host work).

    Args:
        circ (CompiledCircuit): the circuit
        loss_fn (callable): maps the final state tensor to a scalar loss
            (torch ops only: no host synchronisation inside)
        params (torch.Tensor): example parameters (shape and device)
        warmup (int): eager steps on a side stream before capture
    """

    def __init__(self, circ, loss_fn, params, warmup=2):
        self.circ = circ
        self.loss_fn = loss_fn
        self.static_p = torch.as_tensor(params).detach().to(device=circ.device, dtype=torch.float64).clone()
        cur = torch.cuda.current_stream(circ.device)
        side = torch.cuda.Stream(device=circ.device)
        side.wait_stream(cur)
        with torch.cuda.stream(side):
            for _ in range(warmup):
                self._step()
        cur.wait_stream(side)
        torch.cuda.synchronize(circ.device)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.static_loss, self.static_grad = self._step()

    def _step(self):
        p = self.static_p.detach().requires_grad_(True)
        psi = self.circ(p)
        loss = self.loss_fn(psi)
        (g,) = torch.autograd.grad(loss, p)
        return loss.detach(), g

    def __call__(self, params=None):
        """Replay with new parameters (copied into the captured buffer);
        returns (loss, gradient) tensors owned by the graph."""
        if params is not None:
            self.static_p.copy_(params, non_blocking=True)
        self.graph.replay()
        return self.static_loss, self.static_grad
