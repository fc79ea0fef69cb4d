"""State object returned by the GB300 backend: the counterpart of
``BaseFockState`` (reference ``strawberryfields/backends/states.py:477-986``).

Readouts run on the device: probabilities, per-mode photon-number marginals
and single-mode reduced density matrices never form the full density matrix
of a pure state (the reference's ``reduced_dm``/``mean_photon`` build it,
states.py:613-663).  ``ket()``/``dm()`` copy to the host as numpy arrays, like
the reference; ``ket_tensor()`` exposes the device tensor without a copy.
"""

import sys

import numpy as np
import torch

from . import _lib as L


class FockStateGB300:
    """Fock-basis state held on the GPU.

    Args:
        state_data (torch.Tensor): device state tensor (captured as is)
        num_modes (int): number of modes
        pure (bool): ket ([D]*n) or density matrix ([D]*2n, interleaved axes)
        cutoff_dim (int): Fock cutoff D
        mode_names (Sequence[str]): optional mode names
        hbar (float): value of hbar for quadrature readouts (default: the
            frontend's ``strawberryfields.hbar`` when Strawberry Fields is
            imported -- the reference's states always take it from there,
            states.py:53 -- else 2)
    """

    EQ_TOLERANCE = 1e-10

    def __init__(self, state_data, num_modes, pure, cutoff_dim, mode_names=None, hbar=None):
        if hbar is None:
            sfmod = sys.modules.get("strawberryfields")
            hbar = float(getattr(sfmod, "hbar", 2.0)) if sfmod is not None else 2.0
        # same argument order as BaseFockState (states.py:489); state_data is
        # a CUDA tensor ([D]*n pure, [D]*2n mixed) or a host array
        if not torch.is_tensor(state_data):
            state_data = torch.as_tensor(np.asarray(state_data), device="cuda")
        self._tensor = state_data
        self._pure = bool(pure)
        self._modes = num_modes
        self._cutoff = cutoff_dim
        self._hbar = hbar
        self._basis = "fock"
        self._dcode = L.C64 if state_data.dtype == torch.complex64 else L.C128
        if state_data.dtype not in (torch.complex64, torch.complex128):
            self._tensor = state_data.to(torch.complex128)
            self._dcode = L.C128
        if mode_names is None:
            self._modemap = {i: "mode {}".format(i) for i in range(self._modes)}
        else:
            self._modemap = {i: "{}".format(j) for i, j in zip(range(self._modes), mode_names)}
        self._str = "<FockState: num_modes={}, cutoff={}, pure={}, hbar={}>".format(
            self._modes, self._cutoff, self._pure, self._hbar)

    def __str__(self):
        return self._str

    def __eq__(self, other):
        """Equal when the other state is of this type, has the same modes and
        shape, and the density matrices agree within EQ_TOLERANCE
        (states.py:503-526)."""
        if not isinstance(other, type(self)):
            return False
        if self._modes != other._modes or tuple(self._tensor.shape) != tuple(other._tensor.shape):
            return False
        return bool(np.allclose(self.dm(), other.dm(), atol=self.EQ_TOLERANCE, rtol=0))

    __hash__ = object.__hash__

    __repr__ = __str__

    # ----------------------------------------------------------------- basics
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
    def mode_names(self):
        return self._modemap

    @property
    def mode_indices(self):
        return {v: k for k, v in self._modemap.items()}

    @property
    def data(self):
        return self._tensor.cpu().numpy()

    def ket_tensor(self):
        """Device tensor of the ket (no copy); None for mixed states."""
        return self._tensor if self._pure else None

    def ket(self, **kwargs):
        if self._pure:
            return self._tensor.cpu().numpy()
        return None

    def dm(self, **kwargs):
        if not self._pure:
            return self._tensor.cpu().numpy()
        D, n = self._cutoff, self._modes
        dm = torch.empty([D] * (2 * n), dtype=self._tensor.dtype, device=self._tensor.device)
        L.call("fock_mix", n, D, self._dcode, self._tensor.data_ptr(), dm.data_ptr(),
               torch.cuda.current_stream(self._tensor.device).cuda_stream)
        return dm.cpu().numpy()

    # ----------------------------------------------------------------- readouts
    def _probs_tensor(self):
        D, n = self._cutoff, self._modes
        out = torch.empty([D] * n, dtype=torch.float64, device=self._tensor.device)
        L.call("fock_probs", n, D, int(self._pure), self._dcode, self._tensor.data_ptr(), out.data_ptr(),
               torch.cuda.current_stream(self._tensor.device).cuda_stream)
        return out

    def all_fock_probs(self, **kwargs):
        """Probabilities of all Fock basis states (states.py:580)."""
        return self._probs_tensor().cpu().numpy()

    def trace(self, **kwargs):
        if self._modes == 0:  # every mode deleted: the data is the trace itself
            return float(self._tensor.real.item())
        return float(self._probs_tensor().sum().item())

    def fock_prob(self, n, **kwargs):
        """Probability of one Fock basis state (states.py:644)."""
        if len(n) != self._modes:
            raise ValueError("List length should be equal to number of modes")
        if max(n) >= self._cutoff:
            raise ValueError("Can't get distribution beyond truncation level")
        if self._pure:
            v = self._tensor[tuple(n)].item()
            return abs(v) ** 2
        idx = tuple(n[i // 2] for i in range(len(n) * 2))
        return float(self._tensor[idx].real.item())

    def marginals(self):
        """Photon-number distribution of every mode, numpy [n, D] (one device pass per mode)."""
        D, n = self._cutoff, self._modes
        out = torch.empty((n, D), dtype=torch.float64, device=self._tensor.device)
        lib = L.load()
        ws = torch.empty(lib.fock_marginals_workspace_bytes(n, D, int(self._pure), self._dcode),
                         dtype=torch.uint8, device=self._tensor.device)
        L.call("fock_marginals", n, D, int(self._pure), self._dcode, self._tensor.data_ptr(), out.data_ptr(),
               ws.data_ptr(), torch.cuda.current_stream(self._tensor.device).cuda_stream)
        return out.cpu().numpy()

    def mean_photon(self, mode, **kwargs):
        """(mean, variance) of the photon number of one mode (states.py:657)."""
        p = self.marginals()[mode]
        k = np.arange(self._cutoff)
        mean = float(np.sum(k * p))
        var = float(np.sum(k * k * p) - mean ** 2)
        return mean, var

    def _rdm1_dev(self, mode):
        """One mode's reduced density matrix, complex128 device tensor [D, D]."""
        D, n = self._cutoff, self._modes
        out = torch.empty((D, D), dtype=torch.complex128, device=self._tensor.device)
        lib = L.load()
        ws = torch.empty(lib.fock_reduced_dm1_workspace_bytes(n, D, int(self._pure), self._dcode),
                         dtype=torch.uint8, device=self._tensor.device)
        L.call("fock_reduced_dm1", n, D, int(self._pure), self._dcode, mode, self._tensor.data_ptr(),
               out.data_ptr(), ws.data_ptr(), torch.cuda.current_stream(self._tensor.device).cuda_stream)
        return out

    def _rdm1(self, mode):
        return self._rdm1_dev(mode).cpu().numpy()

    def reduced_dm(self, modes, **kwargs):
        """Reduced density matrix (states.py:613).  One mode: device
        contraction; several modes: the kept modes' block of the density
        matrix, interleaved axes like the reference."""
        if isinstance(modes, int):
            modes = [modes]
        modes = list(modes)
        if modes != sorted(modes):
            raise ValueError("The specified modes cannot be duplicated.")
        if len(modes) > self._modes:
            raise ValueError("The number of specified modes cannot be larger than the number of subsystems.")
        if modes == list(range(self._modes)):
            return self.dm()
        if len(modes) == 1:
            return self._rdm1(modes[0])
        return self._reduced_multi(modes)

    def _reduced_multi(self, modes):
        D, n = self._cutoff, self._modes
        k = len(modes)
        rest = [m for m in range(n) if m not in modes]
        if self._pure:
            psi = self._tensor.permute(modes + rest).reshape(D ** k, -1)
            rho = (psi @ psi.conj().T).reshape([D] * (2 * k))
            perm = []
            for i in range(k):
                perm += [i, k + i]
            return rho.permute(perm).to(torch.complex128).cpu().numpy()
        rho = self._tensor
        # trace out the rest, last mode first so axis numbers stay valid
        for m in sorted(rest, reverse=True):
            rho = torch.diagonal(rho, dim1=2 * m, dim2=2 * m + 1).sum(-1)
        return rho.to(torch.complex128).cpu().numpy()

    # ----------------------------------------------------------------- fidelities
    def fidelity(self, other_state, mode, **kwargs):
        rho = self._rdm1(mode)
        return float(np.dot(np.conj(other_state), np.dot(rho, other_state)).real)

    def fidelity_vacuum(self, **kwargs):
        if self._pure:
            return abs(self._tensor.reshape(-1)[0].item()) ** 2
        return float(self._tensor.reshape(-1)[0].real.item())

    def fidelity_coherent(self, alpha_list, **kwargs):
        if not hasattr(alpha_list, "__len__"):
            alpha_list = [alpha_list]
        if len(alpha_list) != self._modes:
            raise ValueError("The number of alpha values must match the number of modes.")
        from math import factorial

        D = self._cutoff
        vecs = [np.array([np.exp(-0.5 * abs(a) ** 2) * a ** k / np.sqrt(factorial(k)) for k in range(D)],
                         dtype=np.complex128) for a in alpha_list]
        dev = self._tensor.device
        if self._pure:
            x = self._tensor.to(torch.complex128)
            for v in vecs:
                x = torch.tensordot(torch.as_tensor(v.conj(), device=dev), x, dims=([0], [0]))
            return abs(x.item()) ** 2
        x = self._tensor.to(torch.complex128)
        for v in vecs:
            vt = torch.as_tensor(v, device=dev)
            x = torch.tensordot(vt.conj(), x, dims=([0], [0]))
            x = torch.tensordot(vt, x, dims=([0], [0]))
        return float(x.real.item())

    # ----------------------------------------------------------------- quadratures
    def quad_expectation(self, mode, phi=0, **kwargs):
        """Mean and variance of the rotated quadrature
        x_phi = x cos(phi) + p sin(phi) = sqrt(hbar/2) (e^{-i phi} a + e^{i phi} a^dagger)
        of one mode (states.py:730 interface), from ladder-operator moments of
        the mode's reduced density matrix rho (built on the device):
        <a> = sum_n sqrt(n) rho[n, n-1], <a^2> = sum_n sqrt(n(n-1)) rho[n, n-2]
        (and their daggers from the other off-diagonals), and
        <a a^dagger + a^dagger a> = sum_n (2n + 1) rho[n, n].  These are the
        moments of the untruncated operators restricted to the cutoff, so the
        top Fock level contributes (2D - 1) hbar/2 to <x_phi^2>, as in the
        reference's quadrature operators."""
        rho = self._rdm1_dev(mode)
        D = self._cutoff
        n = torch.arange(D, dtype=torch.float64, device=rho.device)
        e1, e2 = np.exp(-1j * phi), np.exp(-2j * phi)
        a1 = torch.sum(torch.sqrt(n[1:]) * torch.diagonal(rho, offset=-1))
        a1d = torch.sum(torch.sqrt(n[1:]) * torch.diagonal(rho, offset=1))
        if D > 2:
            w2 = torch.sqrt(n[2:] * n[1:-1])
            a2 = torch.sum(w2 * torch.diagonal(rho, offset=-2))
            a2d = torch.sum(w2 * torch.diagonal(rho, offset=2))
        else:
            a2 = a2d = torch.zeros((), dtype=rho.dtype, device=rho.device)
        sym = torch.sum((2 * n + 1) * torch.diagonal(rho))
        h = self._hbar / 2
        mean = np.sqrt(h) * complex((e1 * a1 + np.conj(e1) * a1d).item()).real
        second = h * complex((e2 * a2 + np.conj(e2) * a2d + sym).item()).real
        return float(mean), float(second - mean ** 2)

    def wigner(self, mode, xvec, pvec):
        """Discretised Wigner function of one mode (states.py:730): array
        [len(pvec), len(xvec)] with entry [i, j] at (xvec[j], pvec[i]),
        evaluated on the device from the mode's reduced density matrix."""
        rho = self._rdm1_dev(mode)
        dev = rho.device
        xv = torch.as_tensor(np.asarray(xvec, dtype=np.float64).reshape(-1), device=dev)
        pv = torch.as_tensor(np.asarray(pvec, dtype=np.float64).reshape(-1), device=dev)
        out = torch.empty((pv.numel(), xv.numel()), dtype=torch.float64, device=dev)
        L.call("fock_wigner", self._cutoff, rho.data_ptr(), xv.data_ptr(), xv.numel(), pv.data_ptr(), pv.numel(),
               float(self._hbar), out.data_ptr(), torch.cuda.current_stream(dev).cuda_stream)
        return out.cpu().numpy()

    def p_quad_values(self, mode, xvec, pvec):
        """p-quadrature distribution on ``pvec`` (states.py:436): the Wigner
        function integrated over ``xvec`` by Simpson's rule."""
        from scipy.integrate import simpson

        W = self.wigner(mode, xvec, pvec)
        return np.array([simpson(W[i, : len(xvec)], x=xvec) for i in range(len(pvec))])

    def x_quad_values(self, mode, xvec, pvec):
        """x-quadrature distribution on ``xvec`` (states.py:456): the Wigner
        function integrated over ``pvec`` by Simpson's rule."""
        from scipy.integrate import simpson

        W = self.wigner(mode, xvec, pvec)
        return np.array([simpson(W[: len(pvec), i], x=pvec) for i in range(len(xvec))])

    def poly_quad_expectation(self, A, d=None, k=0, phi=0, **kwargs):
        """Mean and variance of the quadrature polynomial
        Q = r^T A r + d^T r + k, r = (x_1..x_N, p_1..p_N) rotated by ``phi``
        (x_phi = x cos phi + p sin phi, p_phi = -x sin phi + p cos phi), as
        the reference evaluates it (states.py:806-945): the operators are
        built in the Fock basis with cutoff D + 1, Q and Q^2 formed there and
        truncated to D, then traced against the reduced density matrix of the
        modes the coefficients touch."""
        N, D = self._modes, self._cutoff
        A = np.zeros([2 * N, 2 * N]) if A is None else np.asarray(A)
        if A.shape != (2 * N, 2 * N):
            raise ValueError("Matrix of quadratic coefficients A must be of size 2Nx2N.")
        if not np.allclose(A.T, A):
            raise ValueError("Matrix of quadratic coefficients A must be symmetric.")
        d = np.zeros([2 * N]) if d is None else np.asarray(d)
        if d.shape != (2 * N,):
            raise ValueError("Vector of linear coefficients d must be of length 2N.")
        modes = sorted({int(i) % N for i in A.nonzero()[0]} | {int(i) % N for i in d.nonzero()[0]})
        if not modes:
            return k, 0.0
        km = len(modes)
        dim = D + 1
        a = np.diag(np.sqrt(np.arange(1, dim)), 1)
        x0 = np.sqrt(self._hbar / 2) * (a + a.T)
        p0 = -1j * np.sqrt(self._hbar / 2) * (a - a.T)
        xr = np.cos(phi) * x0 + np.sin(phi) * p0
        pr = -np.sin(phi) * x0 + np.cos(phi) * p0

        def on_mode(op, q):
            out = np.ones((1, 1))
            for j in range(km):
                out = np.kron(out, op if j == q else np.eye(dim))
            return out

        r = [on_mode(xr, q) for q in range(km)] + [on_mode(pr, q) for q in range(km)]
        idx = modes + [N + m for m in modes]
        Aq = A[np.ix_(idx, idx)]
        op = np.zeros((dim ** km, dim ** km), dtype=np.complex128)
        for i in range(2 * km):
            row = sum(Aq[i, j] * r[j] for j in range(2 * km) if Aq[i, j] != 0)
            if not np.isscalar(row):
                op += r[i] @ row
            if d[idx[i]] != 0:
                op += d[idx[i]] * r[i]
        if k != 0:
            op += k * np.eye(dim ** km)
        op2 = op @ op

        def truncate(M):
            return M.reshape([dim] * (2 * km))[(slice(0, D),) * (2 * km)].reshape(D ** km, D ** km)

        rho = np.asarray(self.reduced_dm(modes))
        # interleaved [o0, i0, o1, i1, ...] -> matrix [(o0 o1 ..), (i0 i1 ..)]
        rho = rho.transpose([2 * q for q in range(km)] + [2 * q + 1 for q in range(km)]).reshape(D ** km, D ** km)
        mean = float(np.real(np.trace(truncate(op) @ rho)))
        var = float(np.real(np.trace(truncate(op2) @ rho)) - mean ** 2)
        return mean, var

    def number_expectation(self, modes):
        values = np.arange(self._cutoff)
        mean = self.diagonal_expectation(modes, values)
        var = self.diagonal_expectation(modes, values ** 2) - mean ** 2
        return mean, var

    def parity_expectation(self, modes):
        return self.diagonal_expectation(modes, (-1) ** np.arange(self._cutoff))

    def diagonal_expectation(self, modes, values):
        if len(modes) != len(set(modes)):
            raise ValueError("There can be no duplicates in the modes specified.")
        ps = self._probs_tensor()
        traced = tuple(m for m in range(self._modes) if m not in modes)
        if traced:
            ps = ps.sum(dim=traced)
        vt = torch.as_tensor(np.asarray(values, dtype=np.float64), device=ps.device)
        for _ in modes:
            ps = torch.tensordot(vt, ps, dims=1)
        return float(ps.item())
