"""Device-resident Fock circuit: the GB300 counterpart of the reference's
``strawberryfields/backends/fockbackend/circuit.py`` ``Circuit`` class.

The state lives in HBM as a torch tensor (``[D]*n`` pure, ``[D]*2n`` mixed,
interleaved ket/bra axes) and every update runs through the C-ABI library
(``libfockgb300.so``).  Rotation and Kerr gates are not applied when called:
they accumulate per mode and are folded into the next non-diagonal gate on
that mode (``pre`` phases of ``fock_apply_gate``), or flushed as one diagonal
pass before any readout -- the state crosses HBM once per gate group.
"""

import ctypes
import math
import numbers

import numpy as np
import torch

from . import _lib as L

MAX_MODES = 23  # same limit as the reference (fockbackend/circuit.py:32)


def _dtype_code(dtype):
    if dtype in (torch.complex64, np.complex64, "complex64"):
        return L.C64, torch.complex64
    if dtype in (torch.complex128, np.complex128, "complex128", None):
        return L.C128, torch.complex128
    raise ValueError(f"unsupported dtype {dtype!r}: use complex64 or complex128")


class DeviceCircuit:
    """Truncated Fock-basis simulator state on one GPU.

    Args mirror ``Circuit(num, trunc, pure)`` (reference circuit.py:41);
    ``dtype`` selects complex64 or complex128 storage (gate matrices are built
    in FP64 either way) and ``device`` the CUDA device.
    """

    def __init__(self, num, trunc, pure=True, dtype=torch.complex128, device=None):
        if num < 0:
            raise ValueError("Number of modes must be non-negative -- got {}".format(num))
        if num > MAX_MODES:
            raise ValueError("Fock simulator has a maximum of {} modes".format(MAX_MODES))
        if trunc <= 0:
            raise ValueError("Truncation must be positive -- got {}".format(trunc))
        L.load()
        if not torch.cuda.is_available():
            raise RuntimeError("the GB300 Fock backend needs a CUDA device")
        self._dcode, self._tdtype = _dtype_code(dtype)
        self._device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self._num_modes = num
        self._hbar = 2
        self._ws = torch.empty(0, dtype=torch.uint8, device=self._device)
        self.reset(pure=pure, cutoff_dim=trunc)

    # ------------------------------------------------------------------ utils
    @property
    def dtype(self):
        return self._tdtype

    def _stream(self):
        return torch.cuda.current_stream(self._device).cuda_stream

    def _shape(self, pure=None, n=None):
        pure = self._pure if pure is None else pure
        n = self._num_modes if n is None else n
        return [self._trunc] * (n if pure else 2 * n)

    def _empty(self, pure=None, n=None):
        return torch.empty(self._shape(pure, n), dtype=self._tdtype, device=self._device)

    def _workspace(self, nbytes):
        nbytes = int(nbytes)
        if self._ws.numel() < nbytes:
            self._ws = torch.empty(max(nbytes, 1 << 16), dtype=torch.uint8, device=self._device)
        return self._ws.data_ptr()

    def _clear_pending(self):
        self._theta = [0.0] * self._num_modes
        self._kappa = [0.0] * self._num_modes
        self._ck = []  # (mode_a, mode_b, kappa)

    def _has_pending(self):
        return any(self._theta) or any(self._kappa) or bool(self._ck)

    def _flush(self, modes=None):
        """Apply pending diagonal phases (all modes, or the given modes and any
        cross-Kerr pair touching them) as one pass."""
        if not self._has_pending():
            return
        n, D = self._num_modes, self._trunc
        if modes is None:
            sel = set(range(n))
            cks = self._ck
        else:
            sel = set(modes)
            cks = [c for c in self._ck if c[0] in sel or c[1] in sel]
            for c in cks:
                sel.add(c[0])
                sel.add(c[1])
        ang = np.zeros((n, D))
        k = np.arange(D, dtype=np.float64)
        any_1m = False
        for m in sel:
            if self._theta[m] or self._kappa[m]:
                ang[m] = self._theta[m] * k + self._kappa[m] * k * k
                any_1m = True
        if not any_1m and not cks:
            return
        ang_dev = torch.as_tensor(ang, device=self._device) if any_1m else None
        nck = len(cks)
        ckm = (ctypes_int_array([v for c in cks for v in (c[0], c[1])]) if nck else None)
        ckk = (np.array([c[2] for c in cks], dtype=np.float64) if nck else None)
        out = self._empty()
        L.call("fock_apply_phases", n, D, int(self._pure), self._dcode,
               ang_dev.data_ptr() if ang_dev is not None else None, nck,
               ckm, ckk.ctypes.data_as(L._dp) if nck else None,
               self._state.data_ptr(), out.data_ptr(), self._stream())
        self._state = out
        for m in sel:
            self._theta[m] = 0.0
            self._kappa[m] = 0.0
        self._ck = [c for c in self._ck if c not in cks]

    def _gate(self, kind, p0, p1, mode1, mode2=-1):
        """Apply a non-diagonal gate with pending phases of its modes folded in."""
        n, D = self._num_modes, self._trunc
        two = kind in L.TWO_MODE_KINDS
        # cross-Kerr pending on these modes must act before the gate
        touch = [c for c in self._ck if c[0] in (mode1, mode2) or c[1] in (mode1, mode2)]
        if touch or kind == L.LOSS:
            # the loss superoperator does not commute with Kerr phases: apply
            # pending phases of its mode first instead of folding them in
            self._flush([mode1] + ([mode2] if two else []))
        pre = np.array([self._theta[mode1], self._kappa[mode1],
                        self._theta[mode2] if two else 0.0, self._kappa[mode2] if two else 0.0])
        out = self._empty()
        tmp = None if self._pure or kind == L.LOSS else self._empty()
        ws = self._workspace(L.load().fock_gate_workspace_bytes(kind, D))
        L.call("fock_apply_gate", kind, float(p0), float(p1), mode1, mode2 if two else -1, n, D,
               int(self._pure), self._dcode, pre.ctypes.data_as(L._dp), self._state.data_ptr(),
               out.data_ptr(), tmp.data_ptr() if tmp is not None else None, ws, self._stream())
        self._state = out
        self._theta[mode1] = self._kappa[mode1] = 0.0
        if two:
            self._theta[mode2] = self._kappa[mode2] = 0.0

    # ------------------------------------------------------------------ reset
    def reset(self, pure=None, cutoff_dim=None, num_subsystems=None):
        """Reset to vacuum (reference circuit.py:89-116)."""
        if pure is not None:
            if not isinstance(pure, bool):
                raise ValueError("Argument 'pure' must be either True or False")
            self._pure = pure
        if num_subsystems is not None:
            if not isinstance(num_subsystems, int):
                raise ValueError("Argument 'num_subsystems' must be a positive integer")
            self._num_modes = num_subsystems
        if cutoff_dim is not None:
            if not isinstance(cutoff_dim, int) or cutoff_dim < 1:
                raise ValueError("Argument 'cutoff_dim' must be a positive integer")
            self._trunc = cutoff_dim
        self._clear_pending()
        self._state = self._empty()
        L.call("fock_vacuum", self._num_modes, self._trunc, int(self._pure), self._dcode,
               self._state.data_ptr(), self._stream())

    # ------------------------------------------------------------------ gates
    def phase_shift(self, theta, mode):
        self._theta[mode] += float(theta)

    def kerr_interaction(self, kappa, mode):
        self._kappa[mode] += float(kappa)

    def cross_kerr_interaction(self, kappa, mode1, mode2):
        if mode1 == mode2:
            raise ValueError("cross-Kerr needs two distinct modes")
        self._ck.append((mode1, mode2, float(kappa)))

    def displacement(self, r, phi, mode):
        self._gate(L.DISPLACEMENT, r, phi, mode)

    def squeeze(self, r, theta, mode):
        self._gate(L.SQUEEZE, r, theta, mode)

    def beamsplitter(self, theta, phi, mode1, mode2):
        self._gate(L.BEAMSPLITTER, theta, phi, mode1, mode2)

    def mzgate(self, phi_in, phi_ex, mode1, mode2):
        self._gate(L.MZGATE, phi_in, phi_ex, mode1, mode2)

    def two_mode_squeeze(self, r, theta, mode1, mode2):
        self._gate(L.TWO_MODE_SQUEEZE, r, theta, mode1, mode2)

    def apply_matrix(self, mat, mode):
        """Apply a host-built single-mode matrix (built in FP64)."""
        self._flush([mode])
        mat_dev = torch.as_tensor(np.ascontiguousarray(mat, dtype=np.complex128), device=self._device)
        out = self._empty()
        tmp = None if self._pure else self._empty()
        L.call("fock_apply_matrix1", mat_dev.data_ptr(), mode, self._num_modes, self._trunc, int(self._pure),
               self._dcode, self._state.data_ptr(), out.data_ptr(),
               tmp.data_ptr() if tmp is not None else None, self._stream())
        self._state = out

    def gaussian_gate(self, S, d, modes):
        """General Gaussian unitary with symplectic S (xxpp) and displacement d
        on ``modes`` (the TF backend's Ggate, tfbackend/circuit.py:565 and
        ops.py:457-572, 1115): Choi parameters on the host, the D^m x D^m Fock
        matrix by the Hermite recurrence on the device (FP64), one dense
        k-mode pass (ket and bra passes for a density matrix)."""
        from . import gaussian

        modes = [int(m) for m in modes]
        S = np.asarray(S)
        d = np.asarray(d)
        gaussian.check_gate(S, d)
        m = len(modes)
        if S.shape[0] != 2 * m:
            raise ValueError("The matrix S must act on the given modes (2 x number of modes rows).")
        if len(set(modes)) != m:
            raise ValueError("The specified modes cannot be duplicated.")
        self._flush(modes)
        R, y, C = gaussian.choi_parameters(S, d)
        D = self._trunc
        mat = torch.empty([D] * (2 * m), dtype=torch.complex128, device=self._device)
        Rh = np.ascontiguousarray(R, dtype=np.complex128).view(np.float64)
        yh = np.ascontiguousarray(y, dtype=np.complex128).view(np.float64)
        Ch = np.array([C.real, C.imag], dtype=np.float64)
        lib = L.load()
        L.check(lib.fock_gaussian_gate_matrix(m, D, Rh.ctypes.data, yh.ctypes.data, Ch.ctypes.data,
                                              mat.data_ptr(), self._stream()), "fock_gaussian_gate_matrix")
        ws = torch.empty(int(lib.fock_apply_modes_workspace_bytes(m, D, self._dcode)), dtype=torch.uint8,
                         device=self._device)
        out = self._empty()
        tmp = None if self._pure else self._empty()
        md = (ctypes.c_int * m)(*modes)
        L.check(lib.fock_apply_modes(self._num_modes, D, int(self._pure), self._dcode, m, md, mat.data_ptr(),
                                     self._state.data_ptr(), out.data_ptr(),
                                     tmp.data_ptr() if tmp is not None else None, ws.data_ptr(), self._stream()),
                "fock_apply_modes")
        self._state = out

    def cubic_phase_shift(self, gamma, mode):
        """Cubic phase exp(i gamma x^3 / (3 hbar)) (reference ops.py:296-306:
        the D x D matrix exponential is formed on the host in FP64)."""
        from scipy.linalg import expm

        D = self._trunc
        a = np.diag(np.sqrt(np.arange(1, D, dtype=np.float64)), 1)
        x = (a + a.T) * np.sqrt(self._hbar / 2)
        self.apply_matrix(expm(1j * gamma / (3 * self._hbar) * (x @ x @ x)), mode)

    def loss(self, T, mode):
        """Loss channel (reference circuit.py:617): mixes a pure state first."""
        self._to_mixed()
        self._gate(L.LOSS, T, 0.0, mode)

    # ------------------------------------------------------------------ modes
    def alloc(self, n=1):
        """Append ``n`` vacuum modes after the existing ones (reference
        circuit.py:373-382)."""
        n = int(n)
        if n < 0:
            raise ValueError("Number of modes to add must be non-negative -- got {}".format(n))
        if n == 0:
            return
        if self._num_modes + n > MAX_MODES:
            raise ValueError("Fock simulator has a maximum of {} modes".format(MAX_MODES))
        out = self._empty(n=self._num_modes + n)
        if self._num_modes == 0:
            # every mode was deleted: the state is the scalar trace left over
            L.call("fock_vacuum", n, self._trunc, int(self._pure), self._dcode, out.data_ptr(), self._stream())
            out.mul_(self._state)
        else:
            L.call("fock_append_vacuum", self._num_modes, n, self._trunc, int(self._pure), self._dcode,
                   self._state.data_ptr(), out.data_ptr(), self._stream())
        self._state = out
        self._num_modes += n
        self._theta += [0.0] * n
        self._kappa += [0.0] * n

    def dealloc(self, modes):
        """Trace out ``modes``; the circuit is left in a mixed state over the
        remaining modes, in their order (reference circuit.py:384-391)."""
        modes = sorted({int(m) for m in modes})
        if not modes:
            return
        self._flush()
        n, D = self._num_modes, self._trunc
        keep = [m for m in range(n) if m not in modes]
        if not keep:
            # no modes left: what remains is the trace, as a 0-mode mixed state
            tr = self.probs().sum()
            self._state = tr.to(self._tdtype).reshape(())
            self._pure = False
        elif self._pure:
            # rho_keep = A A^dagger with A = psi as [kept modes, traced modes]
            # (a plain GEMM), then the interleaved (ket, bra) axis order
            k = len(keep)
            a = self._state.permute(keep + modes).reshape(D ** k, -1)
            rho = (a @ a.conj().T).reshape([D] * (2 * k))
            perm = [q + s for q in range(k) for s in (0, k)]
            self._state = rho.permute(perm).contiguous()
            self._pure = False
        else:
            out = self._empty(pure=False, n=len(keep))
            L.call("fock_partial_trace", n, D, self._dcode, len(modes), ctypes_int_array(modes),
                   self._state.data_ptr(), out.data_ptr(), self._stream())
            self._state = out
        self._num_modes = len(keep)
        self._clear_pending()

    # ------------------------------------------------------------------ states
    def _to_mixed(self):
        if not self._pure:
            return
        self._flush()
        dm = self._empty(pure=False)
        L.call("fock_mix", self._num_modes, self._trunc, self._dcode, self._state.data_ptr(), dm.data_ptr(),
               self._stream())
        self._state = dm
        self._pure = False

    def prepare_multimode(self, state, modes):
        """Replace ``modes`` by ``state`` (reference circuit.py:393-473).

        As in the reference, preparing a subset of the modes leaves the circuit
        in a mixed state; preparing all modes replaces the state outright."""
        if isinstance(modes, int):
            modes = [modes]
        modes = list(modes)
        n_sub = len(modes)
        D = self._trunc
        state = np.asarray(state)
        pure_shape = (D,) * n_sub
        mixed_shape = (D,) * (2 * n_sub)
        if state.shape == (D ** n_sub,):
            state = state.reshape(pure_shape)
        elif state.shape == (D ** n_sub, D ** n_sub):
            state = state.reshape(mixed_shape)
        if state.shape not in (pure_shape, mixed_shape):
            raise ValueError("Incorrect shape for state preparation")
        if len(modes) != len(set(modes)):
            raise ValueError("The specified modes cannot appear multiple times.")
        is_pure_in = state.shape == pure_shape
        if n_sub == self._num_modes:
            self._clear_pending()
            # order axes so that state's k-th mode lands on modes[k]
            perm = np.argsort(modes)
            if is_pure_in:
                arr = np.transpose(state, perm)
            else:
                arr = np.transpose(state, [2 * p + i for p in perm for i in (0, 1)])
            self._pure = bool(is_pure_in)
            self._state = torch.as_tensor(np.ascontiguousarray(arr), device=self._device).to(self._tdtype)
            return
        self._to_mixed()
        self._flush()
        if is_pure_in:
            flat = state.reshape(-1)
            sub = np.multiply.outer(flat, flat.conj()).reshape((D,) * (2 * n_sub))
            perm = []
            for i in range(n_sub):
                perm += [i, n_sub + i]
            sub = np.transpose(sub.reshape((D,) * (2 * n_sub)), perm)
        else:
            sub = state
        sub_dev = torch.as_tensor(np.ascontiguousarray(sub, dtype=np.complex128), device=self._device)
        out = self._empty()
        ws = self._workspace(L.load().fock_prepare_workspace_bytes(self._num_modes, D, self._dcode, n_sub))
        mm = ctypes_int_array(modes)
        L.call("fock_prepare_modes", self._num_modes, D, self._dcode, n_sub, mm, sub_dev.data_ptr(),
               self._state.data_ptr(), out.data_ptr(), ws, self._stream())
        self._state = out

    def prepare(self, state, mode):
        """Prepare one mode in ``state``; a mixed circuit receives a
        single-mode ket as its density matrix (reference circuit.py:489-528)."""
        state = np.asarray(state)
        if not self._pure and state.ndim == 1:
            state = np.outer(state, state.conj())
        self.prepare_multimode(state, [mode] if isinstance(mode, int) else mode)

    def prepare_mode_fock(self, n, mode):
        st = np.zeros(self._trunc, dtype=np.complex128)
        if n < self._trunc:
            st[n] = 1.0
        self.prepare(st, mode)

    def gate_matrix(self, kind, p0, p1, cutoff=None):
        """FP64 gate matrix built on the device (dense D x D for single-mode
        kinds, photon-number blocks for two-mode kinds)."""
        D = cutoff or self._trunc
        lib = L.load()
        ne = lib.fock_gate_matrix_entries(kind, D)
        out = torch.empty(ne, dtype=torch.complex128, device=self._device)
        ws = self._workspace(lib.fock_gate_workspace_bytes(kind, D))
        L.call("fock_gate_matrix", kind, float(p0), float(p1), D, out.data_ptr(), None, ws, self._stream())
        return out.reshape(D, D) if kind not in L.TWO_MODE_KINDS + (L.LOSS,) else out

    def prepare_mode_coherent(self, r, phi, mode):
        # D(alpha)|0> is column 0 of the displacement matrix (reference ops.py:391)
        vec = self.gate_matrix(L.DISPLACEMENT, r, phi)[:, 0]
        self.prepare(vec.cpu().numpy(), mode)

    def prepare_mode_squeezed(self, r, theta, mode):
        # S(z)|0> is column 0 of the squeezing matrix (reference ops.py:405)
        vec = self.gate_matrix(L.SQUEEZE, r, theta)[:, 0]
        self.prepare(vec.cpu().numpy(), mode)

    def prepare_mode_displaced_squeezed(self, r_d, phi_d, r_s, phi_s, mode):
        # D(alpha) S(z)|0> (reference ops.py:419): the product runs over an
        # extended cutoff so the truncated amplitudes are exact
        D = self._trunc
        De = min(D + 40, 64)
        s = self.gate_matrix(L.SQUEEZE, r_s, phi_s, De)[:, 0]
        vec = self.gate_matrix(L.DISPLACEMENT, r_d, phi_d, De) @ s
        self.prepare(vec[:D].cpu().numpy(), mode)

    def prepare_mode_gkp(self, theta, phi, epsilon, ampl_cutoff, mode):
        """Finite-energy square-lattice GKP qubit
        cos(theta/2)|0>_gkp + e^{-i phi} sin(theta/2)|1>_gkp (reference
        circuit.py:803 and ops.py:518-599): each logical state is a sum over
        lattice teeth t of displaced squeezed vacua D(a_t) S(r)|0>, with
        a_t = sqrt(pi/2)(2t + mu)/cosh(eps), weight exp(-pi/2 tanh(eps)(2t + mu)^2),
        r = -log(tanh eps)/2, and the teeth |t| <= ceil(sqrt(-log(ampl_cutoff)
        / (4 pi tanh eps))) -- the reference's finite-energy definition.  The
        displaced squeezed vacua are the device-built gate matrices applied
        at an extended cutoff (exact truncated amplitudes up to the tail of
        the squeezed vacuum past it), then normalised."""
        D = self._trunc
        De = 64
        th = math.tanh(epsilon)
        z_max = int(np.ceil(np.sqrt(-0.25 / np.pi * np.log(ampl_cutoff) / th)))
        r = -0.5 * math.log(th)
        sq = self.gate_matrix(L.SQUEEZE, r, 0.0, De)[:, 0]
        kets = []
        for mu in (0, 1):
            v = torch.zeros(D, dtype=torch.complex128, device=self._device)
            for t in range(-z_max, z_max + 1):
                a = math.sqrt(0.5 * np.pi) * (2 * t + mu) / math.cosh(epsilon)
                w = math.exp(-0.5 * np.pi * th * (mu + 2 * t) ** 2)
                disp = self.gate_matrix(L.DISPLACEMENT, abs(a), np.pi if a < 0 else 0.0, De)
                v = v + w * (disp @ sq)[:D]
            kets.append(v)
        ket = math.cos(theta / 2) * kets[0] + math.sin(theta / 2) * np.exp(-1j * phi) * kets[1]
        ket = ket / torch.linalg.vector_norm(ket)
        self.prepare(ket.cpu().numpy(), mode)

    def prepare_mode_thermal(self, nbar, mode):
        D = self._trunc
        if nbar == 0:
            st = np.zeros((D, D), dtype=np.complex128)
            st[0, 0] = 1.0
        else:
            st = np.diag([nbar ** n / (nbar + 1) ** (n + 1) for n in range(D)]).astype(np.complex128)
        self.prepare(st, mode)

    # ------------------------------------------------------------------ readout
    def get_state(self):
        """(device tensor, pure) with all pending phases applied."""
        self._flush()
        return self._state, self._pure

    def norm(self):
        s, pure = self.get_state()
        if self._num_modes == 0:
            return float(s.real.item())
        if pure:
            return float(torch.linalg.vector_norm(s).item())
        return float(self.probs().sum())

    def is_vacuum(self, tol):
        s, pure = self.get_state()
        v = s.reshape(-1)[0].item()
        fid = abs(v) ** 2 if pure else v.real
        return abs(fid - 1) <= tol

    def probs(self):
        """all_fock_probs on the device (float64 tensor [D]*n)."""
        s, pure = self.get_state()
        out = torch.empty([self._trunc] * self._num_modes, dtype=torch.float64, device=self._device)
        L.call("fock_probs", self._num_modes, self._trunc, int(pure), self._dcode, s.data_ptr(), out.data_ptr(),
               self._stream())
        return out

    def marginals(self):
        """Per-mode photon-number distributions, float64 tensor [n, D]."""
        s, pure = self.get_state()
        out = torch.empty((self._num_modes, self._trunc), dtype=torch.float64, device=self._device)
        ws = self._workspace(L.load().fock_marginals_workspace_bytes(self._num_modes, self._trunc, int(pure),
                                                                     self._dcode))
        L.call("fock_marginals", self._num_modes, self._trunc, int(pure), self._dcode, s.data_ptr(),
               out.data_ptr(), ws, self._stream())
        return out

    def reduced_dm1(self, mode):
        """Single-mode reduced density matrix (complex128 [D, D])."""
        s, pure = self.get_state()
        out = torch.empty((self._trunc, self._trunc), dtype=torch.complex128, device=self._device)
        ws = self._workspace(L.load().fock_reduced_dm1_workspace_bytes(self._num_modes, self._trunc, int(pure),
                                                                       self._dcode))
        L.call("fock_reduced_dm1", self._num_modes, self._trunc, int(pure), self._dcode, mode, s.data_ptr(),
               out.data_ptr(), ws, self._stream())
        return out

    def dm(self):
        s, pure = self.get_state()
        if not pure:
            return s
        dm = self._empty(pure=False)
        L.call("fock_mix", self._num_modes, self._trunc, self._dcode, s.data_ptr(), dm.data_ptr(), self._stream())
        return dm

    # ------------------------------------------------------------------ measurement
    def measure_fock(self, modes, select=None, rng=None):
        """Photon-number measurement with projection onto |0> of the measured
        modes (reference circuit.py:623-711)."""
        if select is not None and np.any(np.array(select, dtype=object) == None):  # noqa: E711
            raise NotImplementedError("Post-selection lists must only contain numerical values.")
        D, n = self._trunc, self._num_modes
        if select is not None:
            if len(select) != len(modes):
                raise ValueError("When performing post-selection, the number of "
                                 "selected values (including None) must match the number of measured modes")
            if not all(isinstance(s, int) for s in select):
                raise TypeError("The post-select list elements either be integers or None")
            outcome = list(select)
        else:
            probs = self.probs().cpu().numpy()
            other = tuple(i for i in range(n) if i not in modes)
            dist = probs.sum(axis=other) if other else probs
            # order the remaining axes like `modes` (sorted axes -> requested order)
            srt = sorted(modes)
            dist = np.transpose(dist, [srt.index(m) for m in modes]).ravel()
            dist = dist * ~np.isclose(dist, 0.0)
            rng = rng or np.random
            i = rng.choice(len(dist), p=dist / dist.sum())
            outcome = [int(i // D ** (len(modes) - 1 - k) % D) for k in range(len(modes))]
        self._project_reset(modes, outcome)
        nrm = self.norm()
        if nrm == 0:
            raise ZeroDivisionError("Measurement has zero probability.")
        if self._pure:
            self._state = self._state / nrm
        else:
            self._state = self._state / nrm
        return np.array([outcome])

    def homodyne_pdf(self, phi, mode, q_max=10.0, num_bins=100000):
        """Quadrature distribution of x_phi on ``mode`` on the grid
        ``linspace(-q_max, q_max, num_bins)``, as probabilities per bin (the
        pdf times the bin width; reference circuit.py:734-755): from the mode's
        reduced density matrix rotated by R(-phi), with the Hermite functions
        h_n = H_n / sqrt(2^n n!) by their normalised recurrence.  Returns
        (grid, probabilities) as float64 device tensors."""
        D = self._trunc
        mw = 1.0 / self._hbar
        rho = self.reduced_dm1(mode)
        n = torch.arange(D, dtype=torch.float64, device=self._device)
        ph = torch.exp(-1j * phi * n)
        rho = ph[:, None] * rho * ph.conj()[None, :]
        q = torch.linspace(-q_max, q_max, num_bins, dtype=torch.float64, device=self._device)
        x = math.sqrt(mw) * q
        h = torch.empty((D, num_bins), dtype=torch.float64, device=self._device)
        h[0] = 1.0
        if D > 1:
            h[1] = math.sqrt(2.0) * x
        for k in range(2, D):
            h[k] = math.sqrt(2.0 / k) * x * h[k - 1] - math.sqrt((k - 1) / k) * h[k - 2]
        hc = h.to(torch.complex128)
        dist = torch.sum((rho @ hc) * hc, dim=0).real
        dist = dist * math.sqrt(mw / math.pi) * torch.exp(-mw * q * q) * (q[1] - q[0])
        return q, dist

    def measure_homodyne(self, phi, mode, select=None, rng=None, **kwargs):
        """Homodyne measurement of the quadrature x cos(phi) + p sin(phi) of
        ``mode`` (reference circuit.py:713-801): one sample from the binned
        distribution (``num_bins`` points in [-``max``, ``max``]), or the
        post-selected value ``select``; the mode is then projected with
        |0><x_phi| (x_phi the finite-cutoff quadrature eigenstate
        R(phi) D(alpha) times the infinitely squeezed vacuum) and the state
        renormalised.  Returns [[x]]."""
        D = self._trunc
        mw = 1.0 / self._hbar
        if select is not None:
            if not isinstance(select, numbers.Number):
                raise TypeError("Selected measurement result must be of numeric type.")
            sample = float(select)
        else:
            q, dist = self.homodyne_pdf(phi, mode, kwargs.get("max", 10), kwargs.get("num_bins", 100000))
            probs = dist.cpu().numpy()
            probs = probs / probs.sum()
            probs[np.abs(probs) < 1e-10] = 0
            rng = rng or np.random
            idx = int(np.argmax(rng.multinomial(1, probs / probs.sum())))
            sample = float(q[idx].item())
        # |x_phi> in the truncated Fock basis
        sq = np.zeros(D, dtype=np.complex128)
        for k in range(0, D, 2):
            sq[k] = (-0.5) ** (k // 2) * math.sqrt(math.factorial(k)) / math.factorial(k // 2)
        alpha = sample * math.sqrt(mw / 2)
        disp = self.gate_matrix(L.DISPLACEMENT, abs(alpha), float(np.angle(alpha))).cpu().numpy()
        rot = np.exp(1j * phi * np.arange(D))
        eig = (rot[:, None] * disp) @ sq
        P = np.zeros((D, D), dtype=np.complex128)
        P[0, :] = eig.conj()
        self.apply_matrix(P, mode)
        nrm = self.norm()
        if nrm == 0:
            raise ZeroDivisionError("Measurement has zero probability.")
        self._state = self._state / nrm
        return np.array([[sample]])

    def _project_reset(self, modes, values):
        """Apply |0><x| on each measured mode (reference ops.py:180-205)."""
        self._flush()
        D = self._trunc
        for m, x in zip(modes, values):
            P = np.zeros((D, D), dtype=np.complex128)
            if x < D:
                P[0, x] = 1.0
            self.apply_matrix(P, m)


def ctypes_int_array(vals):
    import ctypes

    arr = (ctypes.c_int * len(vals))(*[int(v) for v in vals])
    return arr
