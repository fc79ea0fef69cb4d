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
    """

    def __init__(self, num_modes, cutoff, gates, n_params, dtype=torch.complex64, device=None, batch=1):
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
        L.check(lib.fock_plan_create_batch(self.num_modes, self.cutoff, 1, self._dcode, arr, len(gates),
                                           self.n_params, self.batch, ctypes.byref(plan)), "fock_plan_create")
        self._plan = plan
        info = L.PlanInfo()
        L.check(lib.fock_plan_get_info(plan, ctypes.byref(info)), "fock_plan_get_info")
        self.info = info
        self.n_gates = len(gates)
        self.shape = [self.cutoff] * self.num_modes
        self._bshape = ([self.batch] if self.batch > 1 else []) + self.shape
        self._ws = torch.empty(int(info.workspace_bytes), dtype=torch.uint8, device=self.device)
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

    def forward_states(self, params, state_in=None, store_all=True):
        """Run the forward sweep; returns the [n_ops, D..] tensor of op outputs
        (the last one is the final state).  With store_all=False only two
        slots are kept and the final state is returned alone."""
        p = self._params(params)
        x = self._vacuum if state_in is None else state_in.to(self.dtype).contiguous()
        n = self.n_ops
        if n == 0:
            return x.clone().unsqueeze(0)
        slots = n if store_all else min(n, 2)
        states = torch.empty([slots] + self._bshape, dtype=self.dtype, device=self.device)
        L.check(L.load().fock_plan_forward(self._plan, p.data_ptr(), x.data_ptr(), states.data_ptr(),
                                           int(store_all), self._ws.data_ptr(), self._stream()),
                "fock_plan_forward")
        if store_all:
            return states
        return states[(n - 1) & 1]

    def backward(self, params, states, grad_state, state_in=None):
        """Adjoint sweep: returns (dL/dparams, dL/dstate_in) given dL/dpsi_final."""
        p = self._params(params)
        x = self._vacuum if state_in is None else state_in.to(self.dtype).contiguous()
        lam = grad_state.to(self.dtype).contiguous().clone()
        tmp = torch.empty_like(lam)
        grads = torch.empty(([self.batch] if self.batch > 1 else []) + [self.n_params], dtype=torch.float64,
                            device=self.device)
        if self.n_ops == 0:
            grads.zero_()
            return grads, lam
        L.check(L.load().fock_plan_backward(self._plan, p.data_ptr(), x.data_ptr(), states.data_ptr(),
                                            lam.data_ptr(), tmp.data_ptr(), grads.data_ptr(),
                                            self._ws.data_ptr(), self._stream()),
                "fock_plan_backward")
        return grads, lam

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
        return states[-1].clone() if circ.n_ops else states[0]

    @staticmethod
    def backward(ctx, grad_out):
        params, states = ctx.saved_tensors
        grads, lam = ctx.circ.backward(params, states, grad_out, ctx.state_in)
        gin = lam if (ctx.state_in is not None and ctx.needs_input_grad[2]) else None
        return grads.to(params.dtype), None, gin
