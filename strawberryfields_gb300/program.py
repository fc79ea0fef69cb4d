"""A Strawberry Fields ``Program`` compiled into a differentiable GB300 circuit.

The reference trains circuits by recording a ``Program`` whose gate arguments
are free parameters (``prog.params(...)``, strawberryfields/program.py:853-900,
``FreeParameter`` in parameters.py:379) and running it on the TF backend
inside a ``GradientTape`` with ``eng.run(prog, args=mapping)`` each step
(examples/quantum_neural_network.py:185-216): every step re-walks the
program, evaluates every parameter (``par_evaluate``, parameters.py:162-231)
and applies gate by gate with TF autodiff.

:class:`ProgramCircuit` records such a program once: it decomposes it with
the ``fock`` compiler, maps every gate to the GB300 gate list, and keeps each
gate argument as a constant, a free parameter (up to the sign a daggered
gate puts on its first argument, ops.py:497-501) or a symbolic expression of
free parameters.  Calling it with the free parameters' values -- a mapping
``name -> value`` like ``eng.run(..., args=...)``, or a tensor in
``free_params`` order -- evaluates the gate arguments with torch ops and runs
the compiled circuit; gradients reach the free parameters through the
hand-written adjoint sweep (:class:`~strawberryfields_gb300.CompiledCircuit`).
"""

import numbers

import numpy as np
import torch

from . import _lib as L
from .autograd import CompiledCircuit

# frontend gate class -> (GB300 gate kind, number of arguments)
GATES = {
    "Dgate": (L.DISPLACEMENT, 2),
    "Sgate": (L.SQUEEZE, 2),
    "Rgate": (L.ROTATION, 1),
    "Kgate": (L.KERR, 1),
    "BSgate": (L.BEAMSPLITTER, 2),
    "MZgate": (L.MZGATE, 2),
    "S2gate": (L.TWO_MODE_SQUEEZE, 2),
    "CKgate": (L.CROSS_KERR, 1),
    "LossChannel": (L.LOSS, 1),
}
# state preparations accepted before the first gate (they set the input state)
PREPARATIONS = ("Vacuum", "Coherent", "Squeezed", "DisplacedSqueezed", "Thermal", "Fock", "Ket", "DensityMatrix")

# sympy function names -> torch, for gate arguments that are expressions of
# free parameters
_TORCH_FUNCS = {
    "sin": torch.sin, "cos": torch.cos, "tan": torch.tan, "exp": torch.exp, "log": torch.log,
    "sqrt": torch.sqrt, "Abs": torch.abs, "sinh": torch.sinh, "cosh": torch.cosh, "tanh": torch.tanh,
    "asin": torch.asin, "acos": torch.acos, "atan": torch.atan, "atan2": torch.atan2,
    "arg": torch.angle, "re": torch.real, "im": torch.imag, "pi": np.pi,
}


def _is_symbolic(v):
    try:
        import sympy
    except ImportError:
        return False
    return isinstance(v, sympy.Basic)


def _free_parameter_name(v):
    """Name of a bare free parameter, else None."""
    cls = type(v).__name__
    if cls == "FreeParameter":
        return v.name
    return None


class ProgramGates:
    """The gate list of a reference ``sf.Program`` and its gate arguments as
    a function of the free parameters (host side: no device needed).

    Args:
        prog (strawberryfields.Program): the program (gates Dgate, Sgate,
            Rgate, Kgate, BSgate, MZgate, S2gate, CKgate, LossChannel, and any
            operation the ``fock`` compiler decomposes into them; state
            preparations only before the first gate)
        batch_size (int): parameter sets per call (None: unbatched)
        compile (bool): decompose with the ``fock`` compiler first (default)
    """

    def __init__(self, prog, batch_size=None, compile=True):
        if compile:
            prog = prog.compile(compiler="fock", warn_connected=False)
        self.num_modes = int(prog.num_subsystems)
        self.free_params = list(prog.free_params.keys())
        self._name_index = {n: i for i, n in enumerate(self.free_params)}
        self.batch_size = batch_size
        gates, slots, preps = [], [], []
        touched = set()
        for cmd in prog.circuit:
            name = type(cmd.op).__name__
            modes = [r.ind for r in cmd.reg]
            if name in PREPARATIONS:
                # a preparation commutes with the gates on other modes before it
                if touched & set(modes):
                    raise NotImplementedError(f"{name} after a gate on its mode: run this program with sf.Engine")
                preps.append((cmd.op, modes))
                continue
            touched |= set(modes)
            if name not in GATES:
                raise NotImplementedError(f"{name} is not supported in a compiled GB300 circuit")
            kind, nargs = GATES[name]
            p = list(cmd.op.p[:nargs])
            if name != "LossChannel":
                if isinstance(p[0], numbers.Number) and p[0] == 0:
                    continue  # the reference skips gates whose first argument is 0 (ops.py:494-497)
                if getattr(cmd.op, "dagger", False):
                    p[0] = -p[0]
            two = kind in L.TWO_MODE_KINDS
            gates.append((kind, modes[0], modes[1] if two else -1, len(slots)))
            slots.extend(p)
        self.gates = gates
        self.n_slots = len(slots)
        self._slots_spec(slots)
        self.preparations = preps
        self.mixed = any(k == L.LOSS for k, _, _, _ in gates) or any(
            type(op).__name__ in ("Thermal", "DensityMatrix") for op, _ in preps)

    # ------------------------------------------------------------------ arguments
    def _slots_spec(self, slots):
        const = np.zeros(len(slots))
        index = np.full(len(slots), -1, dtype=np.int64)
        sign = np.ones(len(slots))
        exprs = []
        for s, v in enumerate(slots):
            if not _is_symbolic(v):
                const[s] = float(np.real(v))
                continue
            name = _free_parameter_name(v)
            neg = _free_parameter_name(-v)
            if name is not None:
                index[s] = self._name_index[name]
            elif neg is not None:
                index[s], sign[s] = self._name_index[neg], -1.0
            else:
                exprs.append((s, v))
        self._const, self._index, self._sign = const, index, sign
        self._exprs = []
        if exprs:
            import sympy

            for s, e in exprs:
                atoms = sorted((a for a in e.free_symbols if _free_parameter_name(a) is not None),
                               key=lambda a: a.name)
                fn = sympy.lambdify(atoms, e, modules=[_TORCH_FUNCS, "math"])
                self._exprs.append((s, [self._name_index[a.name] for a in atoms], fn))
        self._dev_spec = None

    def values(self, args, device):
        """Free-parameter values as a float64 tensor [n_free] (or
        [batch, n_free]) on ``device``."""
        B = self.batch_size
        if isinstance(args, dict):
            vals = []
            for n in self.free_params:
                if n not in args:
                    raise ValueError(f"no value for free parameter '{n}'")
                vals.append(torch.as_tensor(args[n], dtype=torch.float64, device=device))
            if not vals:
                return torch.zeros((B, 0) if B else (0,), dtype=torch.float64, device=device)
            if B:
                vals = [v.expand(B) if v.dim() == 0 else v for v in vals]
                return torch.stack(vals, dim=-1)
            return torch.stack(vals)
        x = torch.as_tensor(args, dtype=torch.float64, device=device)
        want = (B, len(self.free_params)) if B else (len(self.free_params),)
        if B and x.dim() == 1:
            x = x.unsqueeze(0).expand(B, -1)
        if tuple(x.shape) != want:
            raise ValueError(f"expected free-parameter values of shape {want}, got {tuple(x.shape)}")
        return x

    def gate_arguments(self, args, device=None):
        """Every gate's arguments (the compiled circuit's parameter vector) as
        a differentiable torch function of the free parameters."""
        device = torch.device(device) if device is not None else torch.device("cpu")
        x = self.values(args, device)
        if self._dev_spec is None or self._dev_spec[0].device != device:
            self._dev_spec = (torch.as_tensor(self._const, device=device),
                              torch.as_tensor(np.where(self._index < 0, len(self.free_params), self._index),
                                              device=device),
                              torch.as_tensor(self._sign, device=device),
                              torch.as_tensor(self._index >= 0, device=device))
        const, idx, sign, used = self._dev_spec
        pad = torch.zeros(x.shape[:-1] + (1,), dtype=x.dtype, device=x.device)
        xe = torch.cat([x, pad], dim=-1)
        g = torch.where(used, sign * xe[..., idx], const)
        if self._exprs:
            g = g.clone()
            for s, cols, fn in self._exprs:
                val = fn(*[x[..., c] for c in cols])
                g[..., s] = torch.as_tensor(val, dtype=torch.float64, device=device)
        if self.n_slots == 0:
            g = torch.zeros(x.shape[:-1] + (1,), dtype=torch.float64, device=device)
        return g


class ProgramCircuit:
    """A reference ``sf.Program`` as a differentiable function of its free
    parameters on the GPU.

    Args:
        prog (strawberryfields.Program): the program (see :class:`ProgramGates`)
        cutoff_dim (int): Fock cutoff D
        dtype: ``torch.complex64`` (default) or ``torch.complex128`` state
        device: CUDA device
        pure (bool): ket or density matrix; default: a ket unless the program
            contains a loss channel or a mixed preparation
        batch_size (int): run ``batch_size`` parameter sets at once (the TF
            backend's batch axis, tfbackend/circuit.py:129-185): argument
            values of shape ``[batch_size]`` (scalars are broadcast), states
            ``[batch_size, D, ...]``
        checkpoint (int): as for :class:`CompiledCircuit`
        compile (bool): decompose with the ``fock`` compiler first (default)
    """

    def __init__(self, prog, cutoff_dim, dtype=torch.complex64, device=None, pure=None, batch_size=None,
                 checkpoint=1, compile=True):
        self.program = ProgramGates(prog, batch_size=batch_size, compile=compile)
        self.num_modes = self.program.num_modes
        self.cutoff = int(cutoff_dim)
        self.batch_size = batch_size
        self.free_params = self.program.free_params
        self.pure = (not self.program.mixed) if pure is None else bool(pure)
        B = int(batch_size) if batch_size else 1
        self.circuit = CompiledCircuit(self.num_modes, self.cutoff, self.program.gates,
                                       max(self.program.n_slots, 1), dtype=dtype, device=device, batch=B,
                                       checkpoint=checkpoint, pure=self.pure)
        self.device = self.circuit.device
        self._state_in = self._prepare_input() if self.program.preparations else None

    def gate_arguments(self, args):
        return self.program.gate_arguments(args, self.device)

    # ------------------------------------------------------------------ input state
    def _prepare_input(self):
        """Input state from the program's leading preparations, built by the
        interactive backend (numeric arguments only)."""
        from .backend import FockGB300Backend

        b = FockGB300Backend()
        b.begin_circuit(self.num_modes, cutoff_dim=self.cutoff, pure=self.pure,
                        dtype="complex128" if self.circuit.dtype == torch.complex128 else "complex64",
                        device=self.device)
        for op, modes in self.program.preparations:
            if any(_is_symbolic(v) for v in op.p):
                raise NotImplementedError("preparations with free parameters are not differentiable here")
            op._apply(modes, b)
        s, _ = b.circuit.get_state()
        s = s.to(self.circuit.dtype)
        if self.batch_size:
            s = s.unsqueeze(0).expand([int(self.batch_size)] + list(s.shape)).contiguous()
        return s

    # ------------------------------------------------------------------ run
    def __call__(self, args):
        """Final state (ket ``[D]*n`` or density matrix ``[D]*2n``; batched:
        a leading batch axis) as a differentiable function of the free
        parameters."""
        return self.circuit(self.gate_arguments(args), self._state_in)
