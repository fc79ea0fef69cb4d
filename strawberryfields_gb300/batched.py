"""``batch_size`` mode of the backend: B copies of one circuit, each gate with
its own parameters per copy -- the batch axis of the reference's TF backend
(``begin_circuit(..., batch_size=B)``, strawberryfields/backends/tfbackend/
backend.py:84-111; batched parameters and states, tfbackend/circuit.py:129-185;
states with a leading batch axis, tfbackend/states.py).

The state is one device tensor ``[B, D, ..., D]``.  Every gate runs as a
one-gate compiled plan with ``batch = B`` (cached per gate kind and modes):
the kernels index the copy with ``blockIdx.z`` and read that copy's matrix,
built on the device from its own parameters, so a batched gate is one launch
whatever B is.  Preparations and readouts run per copy.
"""

import numpy as np
import torch

from . import _lib as L
from .autograd import CompiledCircuit
from .circuit import DeviceCircuit, _dtype_code
from .states import FockStateGB300


class BatchedDeviceCircuit:
    """``batch_size`` copies of a circuit of ``num`` modes at cutoff
    ``trunc`` (``pure``: kets, else density matrices)."""

    def __init__(self, num, trunc, pure, batch_size, dtype=torch.complex64, device=None):
        if int(batch_size) < 2:
            raise ValueError("batch_size of 1 not supported, please use different batch_size or set batch_size=None")
        L.load()
        self._dcode, self._tdtype = _dtype_code(dtype)
        self._device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self._num_modes = int(num)
        self._trunc = int(trunc)
        self._pure = bool(pure)
        self.batch_size = int(batch_size)
        self._hbar = 2
        self._plans = {}
        self.reset(pure)

    # ------------------------------------------------------------------ helpers
    def _slice_circuit(self, b):
        """A DeviceCircuit holding copy b's state (shares no buffer with the
        batch: its updates are stacked back by _each)."""
        dc = object.__new__(DeviceCircuit)
        dc._dcode, dc._tdtype, dc._device = self._dcode, self._tdtype, self._device
        dc._num_modes, dc._trunc, dc._pure, dc._hbar = self._num_modes, self._trunc, self._pure, self._hbar
        dc._ws = torch.empty(0, dtype=torch.uint8, device=self._device)
        dc._clear_pending()
        dc._state = self._state[b].contiguous()
        return dc

    def _each(self, fn):
        """Run fn(circuit_of_copy_b, b) on every copy and stack the results."""
        outs = []
        pure, num = self._pure, self._num_modes
        for b in range(self.batch_size):
            dc = self._slice_circuit(b)
            fn(dc, b)
            dc._flush()
            outs.append(dc._state)
            pure, num = dc._pure, dc._num_modes
        self._state = torch.stack(outs)
        self._pure, self._num_modes = pure, num

    def _param(self, v):
        """A gate argument as B float64 values (a scalar is broadcast)."""
        t = torch.as_tensor(np.asarray(v, dtype=np.float64) if not torch.is_tensor(v) else v.detach(),
                            dtype=torch.float64, device=self._device).reshape(-1)
        if t.numel() == 1:
            t = t.expand(self.batch_size)
        if t.numel() != self.batch_size:
            raise ValueError(f"parameter with {t.numel()} values for a batch of {self.batch_size}")
        return t

    def _gate(self, kind, params, mode1, mode2=-1):
        key = (kind, mode1, mode2, self._pure, self._num_modes)
        plan = self._plans.get(key)
        if plan is None:
            plan = CompiledCircuit(self._num_modes, self._trunc, [(kind, mode1, mode2, 0)], max(len(params), 1),
                                   dtype=self._tdtype, device=self._device, batch=self.batch_size, pure=self._pure)
            self._plans[key] = plan
        p = torch.stack([self._param(v) for v in params], dim=1).contiguous()
        self._state = plan.forward_states(p, state_in=self._state, store_all=False)

    # ------------------------------------------------------------------ state
    def reset(self, pure=None, cutoff_dim=None, num_subsystems=None):
        if pure is not None:
            self._pure = bool(pure)
        if cutoff_dim is not None:
            self._trunc = int(cutoff_dim)
        if num_subsystems is not None:
            self._num_modes = int(num_subsystems)
        shape = [self.batch_size] + [self._trunc] * (self._num_modes if self._pure else 2 * self._num_modes)
        self._state = torch.zeros(shape, dtype=self._tdtype, device=self._device)
        self._state.view(self.batch_size, -1)[:, 0] = 1.0
        self._plans = {}

    def get_state(self):
        return self._state, self._pure

    def _to_mixed(self):
        if self._pure:
            self._each(lambda dc, b: dc._to_mixed())

    # ------------------------------------------------------------------ gates
    def phase_shift(self, theta, mode):
        self._gate(L.ROTATION, [theta], mode)

    def kerr_interaction(self, kappa, mode):
        self._gate(L.KERR, [kappa], mode)

    def cross_kerr_interaction(self, kappa, mode1, mode2):
        self._gate(L.CROSS_KERR, [kappa], mode1, mode2)

    def displacement(self, r, phi, mode):
        self._gate(L.DISPLACEMENT, [r, phi], mode)

    def squeeze(self, r, theta, mode):
        self._gate(L.SQUEEZE, [r, theta], mode)

    def beamsplitter(self, theta, phi, mode1, mode2):
        self._gate(L.BEAMSPLITTER, [theta, phi], mode1, mode2)

    def mzgate(self, phi_in, phi_ex, mode1, mode2):
        self._gate(L.MZGATE, [phi_in, phi_ex], mode1, mode2)

    def two_mode_squeeze(self, r, theta, mode1, mode2):
        self._gate(L.TWO_MODE_SQUEEZE, [r, theta], mode1, mode2)

    def loss(self, T, mode):
        self._to_mixed()
        self._gate(L.LOSS, [T], mode)

    def _per_copy(self, v, b):
        a = np.asarray(v.detach().cpu() if torch.is_tensor(v) else v)
        return a.reshape(-1)[b] if a.size == self.batch_size and a.size > 1 else a.reshape(-1)[0] if a.size == 1 else a

    def cubic_phase_shift(self, gamma, mode):
        self._each(lambda dc, b: dc.cubic_phase_shift(float(self._per_copy(gamma, b)), mode))

    def gaussian_gate(self, S, d, modes):
        self._each(lambda dc, b: dc.gaussian_gate(S, d, modes))

    # ------------------------------------------------------------------ preparations
    def prepare_mode_fock(self, n, mode):
        self._each(lambda dc, b: dc.prepare_mode_fock(int(self._per_copy(n, b)), mode))

    def prepare_mode_coherent(self, r, phi, mode):
        self._each(lambda dc, b: dc.prepare_mode_coherent(float(self._per_copy(r, b)), float(self._per_copy(phi, b)),
                                                          mode))

    def prepare_mode_squeezed(self, r, theta, mode):
        self._each(lambda dc, b: dc.prepare_mode_squeezed(float(self._per_copy(r, b)),
                                                          float(self._per_copy(theta, b)), mode))

    def prepare_mode_displaced_squeezed(self, r_d, phi_d, r_s, phi_s, mode):
        self._each(lambda dc, b: dc.prepare_mode_displaced_squeezed(
            float(self._per_copy(r_d, b)), float(self._per_copy(phi_d, b)), float(self._per_copy(r_s, b)),
            float(self._per_copy(phi_s, b)), mode))

    def prepare_mode_gkp(self, theta, phi, epsilon, ampl_cutoff, mode):
        self._each(lambda dc, b: dc.prepare_mode_gkp(theta, phi, epsilon, ampl_cutoff, mode))

    def prepare_mode_thermal(self, nbar, mode):
        self._each(lambda dc, b: dc.prepare_mode_thermal(float(self._per_copy(nbar, b)), mode))

    def prepare_multimode(self, state, modes):
        st = np.asarray(state)
        D, k = self._trunc, (len(modes) if not isinstance(modes, int) else 1)
        batched = st.shape[0] == self.batch_size and st.shape[1:] in ((D,) * k, (D,) * (2 * k), (D ** k,),
                                                                      (D ** k, D ** k))
        self._each(lambda dc, b: dc.prepare_multimode(st[b] if batched else st, modes))

    # ------------------------------------------------------------------ modes
    def alloc(self, n=1):
        self._each(lambda dc, b: dc.alloc(n))
        self._plans = {}

    def dealloc(self, modes):
        self._each(lambda dc, b: dc.dealloc(modes))
        self._plans = {}

    def is_vacuum(self, tol):
        flat = self._state.reshape(self.batch_size, -1)[:, 0]
        fid = (flat.abs() ** 2 if self._pure else flat.real).cpu().numpy()
        return np.abs(fid - 1) <= tol


class BatchedFockState:
    """State of a batched circuit: every readout of :class:`FockStateGB300`
    with a leading batch axis (the reference's TF states with
    ``batched=True``)."""

    def __init__(self, data, num_modes, pure, cutoff_dim, mode_names=None, hbar=None):
        self._data = data
        self._states = [FockStateGB300(data[b].contiguous(), num_modes, pure, cutoff_dim, mode_names, hbar)
                        for b in range(data.shape[0])]
        self._modes, self._pure, self._cutoff = num_modes, pure, cutoff_dim
        self._hbar = self._states[0].hbar

    batched = True

    @property
    def data(self):
        """The batched state as a host array ([B, D, ...])."""
        return self._data.cpu().numpy()

    @property
    def mode_names(self):
        return self._states[0].mode_names

    @property
    def mode_indices(self):
        return self._states[0].mode_indices

    @property
    def num_modes(self):
        return self._modes

    @property
    def cutoff_dim(self):
        return self._cutoff

    @property
    def is_pure(self):
        return self._pure

    @property
    def hbar(self):
        return self._hbar

    @property
    def batch_size(self):
        return len(self._states)

    def _map(self, name, *args, **kwargs):
        return [getattr(s, name)(*args, **kwargs) for s in self._states]

    def ket(self, **kwargs):
        return self._data.cpu().numpy() if self._pure else None

    def dm(self, **kwargs):
        return np.stack(self._map("dm"))

    def trace(self, **kwargs):
        return np.array(self._map("trace"))

    def all_fock_probs(self, **kwargs):
        return np.stack(self._map("all_fock_probs"))

    def fock_prob(self, n, **kwargs):
        return np.array(self._map("fock_prob", n))

    def reduced_dm(self, modes, **kwargs):
        return np.stack(self._map("reduced_dm", modes))

    def mean_photon(self, mode, **kwargs):
        r = self._map("mean_photon", mode)
        return np.array([m for m, _ in r]), np.array([v for _, v in r])

    def quad_expectation(self, mode, phi=0, **kwargs):
        r = self._map("quad_expectation", mode, phi)
        return np.array([m for m, _ in r]), np.array([v for _, v in r])

    def poly_quad_expectation(self, A, d=None, k=0, phi=0, **kwargs):
        r = self._map("poly_quad_expectation", A, d, k, phi)
        return np.array([m for m, _ in r]), np.array([v for _, v in r])

    def number_expectation(self, modes):
        r = self._map("number_expectation", modes)
        return np.array([m for m, _ in r]), np.array([v for _, v in r])

    def parity_expectation(self, modes):
        return np.array(self._map("parity_expectation", modes))

    def fidelity(self, other_state, mode, **kwargs):
        return np.array(self._map("fidelity", other_state, mode))

    def fidelity_vacuum(self, **kwargs):
        return np.array(self._map("fidelity_vacuum"))

    def fidelity_coherent(self, alpha_list, **kwargs):
        return np.array(self._map("fidelity_coherent", alpha_list))

    def wigner(self, mode, xvec, pvec):
        return np.stack(self._map("wigner", mode, xvec, pvec))
