"""``fock_gb300``: a Strawberry Fields ``BaseFock`` backend on one GB300 GPU.

Same method names, argument meaning and exceptions as the reference's
``FockBackend`` (``strawberryfields/backends/fockbackend/backend.py:29-329``,
interface ``strawberryfields/backends/base.py:117-626``), so an unchanged
``sf.Engine`` program runs on it::

    import strawberryfields as sf
    from strawberryfields_gb300 import sf_backend
    eng = sf.Engine(sf_backend(), backend_options={"cutoff_dim": 12})

``sf_backend()`` returns an instance of a subclass of the installed
``BaseFock`` (required by ``BaseEngine.__init__``, engine.py:74-76); the
plain :class:`FockGB300Backend` works without Strawberry Fields installed.
Extra ``backend_options``: ``dtype`` (``"complex128"``, the reference's
precision and the default, or ``"complex64"``), ``device``, and
``batch_size`` (B >= 2 copies of the circuit with per-copy gate parameters,
the TF backend's batch axis: strawberryfields_gb300/batched.py).
"""

import numpy as np
import torch

from .circuit import DeviceCircuit
from .states import FockStateGB300


class ModeRegister:
    """External mode labels of a circuit.  A label stays valid until its mode
    is deleted; the internal index of a live label is the number of live
    labels before it, because deleting a mode removes its axes from the
    state and appending adds axes at the end.  (The reference keeps the same
    information as an explicit label -> index list, ``ModeMap`` in
    strawberryfields/backends/base.py:27-115.)"""

    def __init__(self, num_subsystems):
        self._initial = num_subsystems
        self._alive = [True] * num_subsystems

    def reset(self):
        self._alive = [True] * self._initial

    def live(self):
        """Labels of the modes that exist, in order."""
        return [m for m, a in enumerate(self._alive) if a]

    def internal(self, modes):
        """Internal indices of live labels (int or list); ``ValueError`` for
        labels out of range or deleted."""
        single = isinstance(modes, (int, np.integer))
        ms = [modes] if single else list(modes)
        if not ms or any(not isinstance(m, (int, np.integer)) or not 0 <= m < len(self._alive)
                         or not self._alive[m] for m in ms):
            raise ValueError("The specified modes are not valid.")
        out = [sum(self._alive[:m]) for m in ms]
        return out[0] if single else out

    def append(self, n):
        self._alive += [True] * n

    def remove(self, modes):
        for m in modes:
            self._alive[m] = False


class FockGB300Backend:
    """GB300-native Fock backend (see module docstring)."""

    short_name = "fock_gb300"
    circuit_spec = "fock"
    compiler = "fock"
    _state_cls = FockStateGB300

    def __init__(self):
        self._supported = {"mixed_states": True, "fock_basis": True}
        self._init_modes = None
        self._modes = None
        self.circuit = None
        self._options = {}

    def __str__(self):
        return self.__class__.__name__

    def supports(self, name):
        return self._supported.get(name, False)

    # ----------------------------------------------------------------- modes
    def _remap_modes(self, modes):
        return self._modes.internal(modes)

    def begin_circuit(self, num_subsystems, **kwargs):
        cutoff_dim = kwargs.get("cutoff_dim", None)
        pure = kwargs.get("pure", True)
        if cutoff_dim is None:
            raise ValueError("Argument 'cutoff_dim' must be passed to the Fock backend")
        if not isinstance(cutoff_dim, int):
            raise ValueError("Argument 'cutoff_dim' must be a positive integer")
        if not isinstance(num_subsystems, int):
            raise ValueError("Argument 'num_subsystems' must be a positive integer")
        if not isinstance(pure, bool):
            raise ValueError("Argument 'pure' must be either True or False")
        dtype = kwargs.get("dtype", "complex128")
        if dtype in (np.complex64, torch.complex64):
            dtype = "complex64"
        if dtype in (np.complex128, torch.complex128):
            dtype = "complex128"
        batch_size = kwargs.get("batch_size", None)
        self._options = {"dtype": dtype, "device": kwargs.get("device", None), "batch_size": batch_size}
        self._init_modes = num_subsystems
        if batch_size is not None:
            from .batched import BatchedDeviceCircuit

            self.circuit = BatchedDeviceCircuit(num_subsystems, cutoff_dim, pure, batch_size, dtype=dtype,
                                                device=self._options["device"])
        else:
            self.circuit = DeviceCircuit(num_subsystems, cutoff_dim, pure, dtype=dtype,
                                         device=self._options["device"])
        self._modes = ModeRegister(num_subsystems)

    def add_mode(self, n=1, **kwargs):
        """Append ``n`` vacuum modes (reference fockbackend/backend.py:130)."""
        self.circuit.alloc(n)
        self._modes.append(int(n))

    def del_mode(self, modes):
        """Trace out ``modes``; their labels become invalid (reference
        fockbackend/backend.py:134)."""
        if isinstance(modes, (int, np.integer)):
            modes = [modes]
        self.circuit.dealloc(self._modes.internal(modes))
        self._modes.remove(modes)

    def get_modes(self):
        return self._modes.live()

    def reset(self, pure=True, **kwargs):
        cutoff = kwargs.get("cutoff_dim", self.circuit._trunc)
        self._modes.reset()
        self.circuit.reset(pure, num_subsystems=self._init_modes, cutoff_dim=cutoff)

    def get_cutoff_dim(self):
        return self.circuit._trunc

    # ----------------------------------------------------------------- preparations
    def prepare_vacuum_state(self, mode):
        self.circuit.prepare_mode_fock(0, self._remap_modes(mode))

    def prepare_coherent_state(self, r, phi, mode):
        self.circuit.prepare_mode_coherent(r, phi, self._remap_modes(mode))

    def prepare_squeezed_state(self, r, phi, mode):
        self.circuit.prepare_mode_squeezed(r, phi, self._remap_modes(mode))

    def prepare_displaced_squeezed_state(self, r_d, phi_d, r_s, phi_s, mode):
        self.circuit.prepare_mode_displaced_squeezed(r_d, phi_d, r_s, phi_s, self._remap_modes(mode))

    def prepare_thermal_state(self, nbar, mode):
        self.circuit.prepare_mode_thermal(nbar, self._remap_modes(mode))

    def prepare_fock_state(self, n, mode):
        self.circuit.prepare_mode_fock(n, self._remap_modes(mode))

    def prepare_gkp(self, state, epsilon, ampl_cutoff, representation="real", shape="square", mode=None):
        """Finite-energy GKP qubit state [theta, phi] on ``mode`` (reference
        fockbackend/backend.py:297-329)."""
        if representation == "complex":
            raise NotImplementedError("The complex description of GKP is not implemented")
        if shape != "square":
            raise NotImplementedError("Only square GKP are implemented for now")
        theta, phi = state[0], state[1]
        self.circuit.prepare_mode_gkp(theta, phi, epsilon, ampl_cutoff, self._remap_modes(mode))

    def prepare_ket_state(self, state, modes):
        self.circuit.prepare_multimode(np.asarray(state), self._remap_modes(modes))

    def prepare_dm_state(self, state, modes):
        self.circuit.prepare_multimode(np.asarray(state), self._remap_modes(modes))

    # ----------------------------------------------------------------- gates
    def rotation(self, phi, mode):
        self.circuit.phase_shift(phi, self._remap_modes(mode))

    def displacement(self, r, phi, mode):
        self.circuit.displacement(r, phi, self._remap_modes(mode))

    def squeeze(self, r, phi, mode):
        self.circuit.squeeze(r, phi, self._remap_modes(mode))

    def two_mode_squeeze(self, r, phi, mode1, mode2):
        self.circuit.two_mode_squeeze(r, phi, self._remap_modes(mode1), self._remap_modes(mode2))

    def beamsplitter(self, theta, phi, mode1, mode2):
        self.circuit.beamsplitter(theta, phi, self._remap_modes(mode1), self._remap_modes(mode2))

    def mzgate(self, phi_in, phi_ex, mode1, mode2):
        self.circuit.mzgate(phi_in, phi_ex, self._remap_modes(mode1), self._remap_modes(mode2))

    def kerr_interaction(self, kappa, mode):
        self.circuit.kerr_interaction(kappa, self._remap_modes(mode))

    def cross_kerr_interaction(self, kappa, mode1, mode2):
        self.circuit.cross_kerr_interaction(kappa, self._remap_modes(mode1), self._remap_modes(mode2))

    def cubic_phase(self, gamma, mode):
        self.circuit.cubic_phase_shift(gamma, self._remap_modes(mode))

    def loss(self, T, mode):
        self.circuit.loss(T, self._remap_modes(mode))

    def gaussian_gate(self, S, d, *modes):
        """N-mode Gaussian gate (the TF backend's gaussian_gate,
        tfbackend/backend.py:231); S symplectic (xxpp), d displacements."""
        self.circuit.gaussian_gate(S, d, self._remap_modes(list(modes)))

    # ----------------------------------------------------------------- measurement
    def _no_batch(self, what):
        if self._options.get("batch_size") is not None:
            raise NotImplementedError(f"{what} is not supported with batch_size")

    def measure_fock(self, modes, shots=1, select=None, **kwargs):
        self._no_batch("measure_fock")
        if shots != 1:
            raise NotImplementedError(
                "fock_gb300 backend currently does not support shots != 1 for Fock measurement")
        return self.circuit.measure_fock(self._remap_modes(modes), select=select)

    def measure_homodyne(self, phi, mode, shots=1, select=None, **kwargs):
        """Homodyne measurement (reference fockbackend/backend.py:184-198).

        Keyword Args:
            num_bins (int): bins of the sampled distribution (default 100000)
            max (float): the distribution is binned on [-max, max] (default 10)
        """
        self._no_batch("measure_homodyne")
        if shots != 1:
            raise NotImplementedError("fock backend currently does not support shots != 1 for homodyne measurement")
        return self.circuit.measure_homodyne(phi, self._remap_modes(mode), select=select, **kwargs)

    def is_vacuum(self, tol=0.0, **kwargs):
        return self.circuit.is_vacuum(tol)

    # ----------------------------------------------------------------- state
    def state(self, modes=None, **kwargs):
        """Current state; ``modes`` selects a reduced (mixed) state
        (reference fockbackend/backend.py:209-264)."""
        s, pure = self.circuit.get_state()
        num = self.circuit._num_modes
        cutoff = self.circuit._trunc
        if self._options.get("batch_size") is not None:
            return self._batched_state(s, pure, num, cutoff, modes)
        if modes is None:
            names = ["q[{}]".format(i) for i in self.get_modes()]
            return self._state_cls(s, num, pure, cutoff, names)
        if isinstance(modes, int):
            modes = [modes]
        red = self._reduce(FockStateGB300(s, num, pure, cutoff), modes, num, cutoff)
        names = ["q[{}]".format(i) for i in np.array(self.get_modes())[modes]]
        t = torch.as_tensor(np.ascontiguousarray(red), device=s.device).to(s.dtype)
        return self._state_cls(t, len(modes), False, cutoff, names)

    def _batched_state(self, s, pure, num, cutoff, modes):
        from .batched import BatchedFockState

        if modes is None:
            return BatchedFockState(s, num, pure, cutoff, ["q[{}]".format(i) for i in self.get_modes()])
        single = [self._state_cls(s[b].contiguous(), num, pure, cutoff) for b in range(s.shape[0])]
        if isinstance(modes, int):
            modes = [modes]
        red = torch.stack([torch.as_tensor(np.asarray(
            FockGB300Backend._reduce(st, modes, num, cutoff)), device=s.device) for st in single]).to(s.dtype)
        return BatchedFockState(red, len(modes), False, cutoff)

    @staticmethod
    def _reduce(full, modes, num, cutoff):
        """Reduced density matrix of ``modes`` (in the given order,
        interleaved axes) of one state."""
        if len(modes) != len(set(modes)):
            raise ValueError("The specified modes cannot be duplicated.")
        if len(modes) > num:
            raise ValueError("The number of specified modes cannot be larger than the number of subsystems.")
        srt = sorted(modes)
        red = full.reduced_dm(srt) if srt != list(range(num)) else full.dm()
        red = np.asarray(red).reshape([cutoff] * (2 * len(modes)))
        if modes != srt:
            perm = np.argsort(modes)
            idx = [2 * x + i for x in perm for i in (0, 1)]
            red = np.transpose(red, np.argsort(idx))
        return red


_SF_CLASS = None


def sf_backend():
    """A ``fock_gb300`` backend instance that is also a ``BaseFock`` of the
    installed Strawberry Fields, for ``sf.Engine(sf_backend(), ...)``."""
    global _SF_CLASS
    if _SF_CLASS is None:
        from strawberryfields.backends.base import BaseFock  # pylint: disable=import-outside-toplevel
        from strawberryfields.backends.states import BaseFockState  # pylint: disable=import-outside-toplevel

        # results carry the state only if it is a BaseState (strawberryfields/result.py)
        state_cls = type("FockStateGB300", (FockStateGB300, BaseFockState), {})
        _SF_CLASS = type("FockGB300Backend", (FockGB300Backend, BaseFock), {"_state_cls": state_cls})
    return _SF_CLASS()


def register():
    """Make ``sf.Engine("fock_gb300")`` resolve to this backend."""
    from strawberryfields import backends  # pylint: disable=import-outside-toplevel

    sf_backend()
    backends.local_backends[FockGB300Backend.short_name] = _SF_CLASS
    return _SF_CLASS
