"""CPU oracle for the Fock-basis hot path -- TEST INFRASTRUCTURE ONLY.

This module is the checker, never the product: only ``tests/``, the smoke check
in ``__graft_entry__`` and the CPU-baseline leg of ``bench.py`` may import it.
The product path (``strawberryfields_gb300``) never calls into it and fails
loudly when its CUDA library is missing.

What it restates (complex128 / FP64 throughout, like the reference):

* gate matrices of ``strawberryfields/backends/fockbackend/ops.py``
  (``displacement`` :219, ``squeezing`` :238, ``two_mode_squeeze`` :257,
  ``kerr`` :274, ``cross_kerr`` :284, ``phase`` :309, ``beamsplitter`` :318,
  ``mzgate`` :332, ``lossChannel`` :471).  The five non-diagonal builders call
  the third-party ``thewalrus.fock_gradients`` (pinned ``thewalrus==0.22.0`` in
  the reference's ``requirements.txt:12``), which is not vendored; they are
  restated here from the gates' ladder-operator definitions
  (``strawberryfields/ops.py`` Dgate :1497, Sgate :1612, BSgate :1864,
  S2gate :2036, MZgate :1951) as exact matrix elements of the infinite
  operator, truncated to the cutoff -- the convention the reference's analytic
  tests pin (coherent, squeezed, TMSV and beamsplitter known answers);
* the state updates of ``strawberryfields/backends/fockbackend/circuit.py``
  (``apply_gate_BLAS`` :118, ``apply_twomode_gate`` :219,
  ``_apply_two_mode_passive`` :307, ``_apply_S2`` :338, ``_apply_channel`` :65)
  and ``ops.mix`` :110, written as ``numpy.tensordot`` contractions instead of
  the reference's per-fibre Python loops (same arithmetic, same index order);
* readouts of ``strawberryfields/backends/states.py`` (``all_fock_probs`` :580,
  ``fock_prob`` :644, ``reduced_dm`` :613, ``mean_photon`` :657) computed from
  marginals instead of the full density matrix, and ``wigner`` :730;
* the TF backend's Gaussian gate (``tfbackend/ops.py:457-572``): ``choi_trick``
  and the renormalised multidimensional Hermite tensor of the third-party
  thewalrus (not vendored; restated from its recurrence), pinned against the
  exact single- and two-mode gate matrices.

Parity of these restatements is pinned by ``tests/test_oracle.py`` against
``scipy.linalg.expm`` of each gate generator, against the reference's own
known-answer formulas, and against golden vectors produced by the reference's
``Circuit`` class itself (``tests/golden/make_golden.py``).

Index conventions (reference ``fockbackend/backend.py:50-56``, ``ops.py:110``):
pure states are ``[m0, m1, ...]`` (mode 0 slowest), mixed states interleave
``[ket0, bra0, ket1, bra1, ...]``; two-mode gate tensors are
``mat[out1, in1, out2, in2]``.
"""

import math

import numpy as np

CDT = np.complex128


# ---------------------------------------------------------------------------
# single-mode gate matrices
# ---------------------------------------------------------------------------

def displacement(r, phi, D):
    """<m|D(r e^{i phi})|n> truncated to D (reference fockbackend/ops.py:219).

    Column recurrence from ``a D(alpha) = D(alpha) (a + alpha)``:
    ``sqrt(m+1) D[m+1,n] = sqrt(n) D[m,n-1] + alpha D[m,n]`` with the first row
    ``D[0,n] = exp(-r^2/2) (-conj(alpha))^n / sqrt(n!)``.  Only lower indices
    are used, so the truncated entries are exact.
    """
    alpha = r * np.exp(1j * phi)
    M = np.zeros((D, D), dtype=CDT)
    n = np.arange(D)
    sq = np.sqrt(np.arange(D, dtype=np.float64))
    row0 = np.empty(D, dtype=CDT)
    row0[0] = np.exp(-0.5 * r * r)
    for k in range(1, D):
        row0[k] = row0[k - 1] * (-np.conj(alpha)) / sq[k]
    M[0] = row0
    for m in range(D - 1):
        prev = np.zeros(D, dtype=CDT)
        prev[1:] = M[m, :-1] * sq[1:]
        M[m + 1] = (prev + alpha * M[m]) / np.sqrt(m + 1.0)
    del n
    return M


def grad_displacement(r, phi, D):
    """(dD/dr, dD/dphi), exact on the truncated block.

    ``d/dphi D[m,n] = i (m-n) D[m,n]`` (D(r e^{i phi}) = R(phi) D(r) R(-phi));
    ``d/dr D[m,n] = e^{i phi} sqrt(m) D[m-1,n] - e^{-i phi} sqrt(n) D[m,n-1] - r D[m,n]``
    (derivative of the generator form, with the upper neighbour eliminated by
    the column recurrence).  Same quantities as the reference's TF gradient
    ``tfbackend/ops.py:318-332`` obtains from thewalrus ``grad_displacement``.
    """
    M = displacement(r, phi, D)
    idx = np.arange(D)
    dphi = 1j * (idx[:, None] - idx[None, :]) * M
    sq = np.sqrt(idx.astype(np.float64))
    up = np.zeros_like(M)
    up[1:] = sq[1:, None] * M[:-1]
    left = np.zeros_like(M)
    left[:, 1:] = sq[None, 1:] * M[:, :-1]
    dr = np.exp(1j * phi) * up - np.exp(-1j * phi) * left - r * M
    return dr, dphi


def _squeezing_ext(r, phi, D):
    """<m|S(r e^{i phi})|n> for m, n < D (exact entries, cutoff independent)."""
    c, s, t = np.cosh(r), np.sinh(r), np.tanh(r)
    eip = np.exp(1j * phi)
    M = np.zeros((D, D), dtype=CDT)
    M[0, 0] = 1.0 / np.sqrt(c)
    for m in range(2, D, 2):
        M[m, 0] = -eip * t * np.sqrt((m - 1.0) / m) * M[m - 2, 0]
    sq = np.sqrt(np.arange(D + 1, dtype=np.float64))
    for n in range(D - 1):
        # S[m,n+1] = (sqrt(m) S[m-1,n] + e^{-i phi} s sqrt(n) S[m,n-1]) / (c sqrt(n+1))
        col = np.zeros(D, dtype=CDT)
        col[1:] = sq[1:D] * M[:-1, n]
        if n >= 1:
            col += np.conj(eip) * s * sq[n] * M[:, n - 1]
        M[:, n + 1] = col / (c * sq[n + 1])
    return M


def squeezing(r, phi, D):
    """<m|S(r e^{i phi})|n>, S(z) = exp((z* a^2 - z a^dag^2)/2) (reference ops.py:238).

    From ``a^dag S = S (c a^dag - e^{-i phi} s a)``:
    ``S[m,n+1] = (sqrt(m) S[m-1,n] + e^{-i phi} s sqrt(n) S[m,n-1]) / (c sqrt(n+1))``,
    seeded by the squeezed-vacuum column ``S[m,0]``.
    """
    return _squeezing_ext(r, phi, D)


def grad_squeezing(r, phi, D):
    """(dS/dr, dS/dphi): ``dS/dr = G S`` with ``G = (e^{-i phi} a^2 - e^{i phi} a^dag^2)/2``
    (evaluated on the cutoff-(D+2) matrix, then truncated, which is exact) and
    ``dS/dphi[m,n] = i (m-n)/2 S[m,n]``."""
    E = _squeezing_ext(r, phi, D + 2)
    a = np.diag(np.sqrt(np.arange(1, D + 2, dtype=np.float64)), 1)
    a2 = a @ a
    G = 0.5 * (np.exp(-1j * phi) * a2 - np.exp(1j * phi) * a2.T)
    dr = (G @ E)[:D, :D]
    S = E[:D, :D]
    idx = np.arange(D)
    dphi = 0.5j * (idx[:, None] - idx[None, :]) * S
    return dr, dphi


def phase(theta, D):
    """R(theta) = exp(i theta n) as a diagonal matrix (reference ops.py:309)."""
    return np.diag(np.exp(1j * theta * np.arange(D))).astype(CDT)


def kerr(kappa, D):
    """K(kappa) = exp(i kappa n^2) (reference ops.py:274)."""
    n = np.arange(D)
    return np.diag(np.exp(1j * kappa * n**2)).astype(CDT)


# ---------------------------------------------------------------------------
# two-mode gate matrices, SF order mat[out1, in1, out2, in2]
# ---------------------------------------------------------------------------

def beamsplitter(theta, phi, D):
    """<m,p|B(theta,phi)|n,q> as ``mat[m,n,p,q]`` (reference ops.py:318).

    From ``B^dag a1 B = t a1 - r* a2`` and ``B^dag a2 B = t a2 + r a1``
    (``ops.py:1892-1893``, t = cos theta, r = e^{i phi} sin theta):
    ``sqrt(m+1) B[m+1,n,p,q] = t sqrt(n) B[m,n-1,p,q] - r* sqrt(q) B[m,n,p,q-1]``,
    ``sqrt(p+1) B[m,n,p+1,q] = t sqrt(q) B[m,n,p,q-1] + r sqrt(n) B[m,n-1,p,q]``,
    seeded by ``B[0,n,0,q] = delta_{n0} delta_{q0}``.
    """
    t = np.cos(theta)
    rr = np.exp(1j * phi) * np.sin(theta)
    sq = np.sqrt(np.arange(D, dtype=np.float64))
    B = np.zeros((D, D, D, D), dtype=CDT)  # [m, n, p, q]
    B[0, 0, 0, 0] = 1.0
    # rows with p = 0, increasing m
    for m in range(D - 1):
        cur = B[m, :, 0, :]  # [n, q]
        nxt = np.zeros((D, D), dtype=CDT)
        nxt[1:, :] += t * sq[1:, None] * cur[:-1, :]
        nxt[:, 1:] -= np.conj(rr) * sq[None, 1:] * cur[:, :-1]
        B[m + 1, :, 0, :] = nxt / np.sqrt(m + 1.0)
    for p in range(D - 1):
        cur = B[:, :, p, :]  # [m, n, q]
        nxt = np.zeros((D, D, D), dtype=CDT)
        nxt[:, :, 1:] += t * sq[None, None, 1:] * cur[:, :, :-1]
        nxt[:, 1:, :] += rr * sq[None, 1:, None] * cur[:, :-1, :]
        B[:, :, p + 1, :] = nxt / np.sqrt(p + 1.0)
    return B


def grad_beamsplitter(theta, phi, D):
    """(dB/dtheta, dB/dphi): ``dB/dtheta = G B`` with
    ``G = e^{i phi} a1 a2^dag - e^{-i phi} a1^dag a2`` on the cutoff-(D+1)
    tensor, and ``dB/dphi[m,n,p,q] = i (p-q) B`` (B(theta,phi) =
    R2(phi) B(theta,0) R2(-phi))."""
    E = beamsplitter(theta, phi, D + 1)
    sq = np.sqrt(np.arange(D + 1, dtype=np.float64))
    # (a1 a2^dag B)[m,n,p,q] = sqrt(m+1) sqrt(p) B[m+1,n,p-1,q]
    t1 = np.zeros((D, D, D, D), dtype=CDT)
    t1[:, :, 1:, :] = (sq[1:D + 1, None, None, None] * sq[None, None, 1:D, None]
                       * E[1:D + 1, :D, 0:D - 1, :D])
    # (a1^dag a2 B)[m,n,p,q] = sqrt(m) sqrt(p+1) B[m-1,n,p+1,q]
    t2 = np.zeros((D, D, D, D), dtype=CDT)
    t2[1:, :, :, :] = (sq[1:D, None, None, None] * sq[None, None, 1:D + 1, None]
                       * E[0:D - 1, :D, 1:D + 1, :D])
    dth = np.exp(1j * phi) * t1 - np.exp(-1j * phi) * t2
    B = E[:D, :D, :D, :D]
    idx = np.arange(D)
    dphi = 1j * (idx[None, None, :, None] - idx[None, None, None, :]) * B
    return dth, dphi


def two_mode_squeeze(r, phi, D):
    """<m,p|S2(r e^{i phi})|n,q> as ``mat[m,n,p,q]`` (reference ops.py:257).

    ``S2 = exp(z a1^dag a2^dag - z* a1 a2)``; from
    ``a1^dag S2 = S2 (c a1^dag + e^{-i phi} s a2)`` and the mirror identity:
    ``T[m,n+1,p,q] = (sqrt(m) T[m-1,n,p,q] - e^{-i phi} s sqrt(q) T[m,n,p,q-1]) / (c sqrt(n+1))``,
    ``T[m,n,p,q+1] = (sqrt(p) T[m,n,p-1,q] - e^{-i phi} s sqrt(n) T[m,n-1,p,q]) / (c sqrt(q+1))``,
    seeded by ``T[m,0,p,0] = delta_{mp} (e^{i phi} tanh r)^m / cosh r``.
    """
    c, s = np.cosh(r), np.sinh(r)
    emp = np.exp(-1j * phi)
    sq = np.sqrt(np.arange(D, dtype=np.float64))
    T = np.zeros((D, D, D, D), dtype=CDT)
    lam = np.exp(1j * phi) * np.tanh(r)
    for m in range(D):
        T[m, 0, m, 0] = lam**m / c
    # increase q with n = 0
    for q in range(D - 1):
        cur = T[:, 0, :, q]  # [m, p]
        nxt = np.zeros((D, D), dtype=CDT)
        nxt[:, 1:] = sq[None, 1:] * cur[:, :-1]
        T[:, 0, :, q + 1] = nxt / (c * np.sqrt(q + 1.0))
    # increase n for all q
    for n in range(D - 1):
        cur = T[:, n, :, :]  # [m, p, q]
        nxt = np.zeros((D, D, D), dtype=CDT)
        nxt[1:, :, :] += sq[1:, None, None] * cur[:-1, :, :]
        nxt[:, :, 1:] -= emp * s * sq[None, None, 1:] * cur[:, :, :-1]
        T[:, n + 1, :, :] = nxt / (c * np.sqrt(n + 1.0))
    return T


def grad_two_mode_squeeze(r, phi, D):
    """(dT/dr, dT/dphi): ``dT/dr = G T`` with
    ``G = e^{i phi} a1^dag a2^dag - e^{-i phi} a1 a2`` on the cutoff-(D+1)
    tensor, ``dT/dphi[m,n,p,q] = i (m-n) T``."""
    E = two_mode_squeeze(r, phi, D + 1)
    sq = np.sqrt(np.arange(D + 1, dtype=np.float64))
    t1 = np.zeros((D, D, D, D), dtype=CDT)  # a1^dag a2^dag T: sqrt(m) sqrt(p) T[m-1,n,p-1,q]
    t1[1:, :, 1:, :] = (sq[1:D, None, None, None] * sq[None, None, 1:D, None]
                        * E[0:D - 1, :D, 0:D - 1, :D])
    t2 = np.zeros((D, D, D, D), dtype=CDT)  # a1 a2 T: sqrt(m+1) sqrt(p+1) T[m+1,n,p+1,q]
    t2[:, :, :, :] = (sq[1:D + 1, None, None, None] * sq[None, None, 1:D + 1, None]
                      * E[1:D + 1, :D, 1:D + 1, :D])
    dr = np.exp(1j * phi) * t1 - np.exp(-1j * phi) * t2
    T = E[:D, :D, :D, :D]
    idx = np.arange(D)
    dphi = 1j * (idx[:, None, None, None] - idx[None, :, None, None]) * T
    return dr, dphi


def _compose2(A, B):
    """(A B)[m,n,p,q] = sum_{k,l} A[m,k,p,l] B[k,n,l,q] for SF-order tensors."""
    return np.einsum("mkpl,knlq->mnpq", A, B)


def mzgate(phi_in, phi_ex, D):
    """MZ(phi_in, phi_ex) = BS(pi/4,pi/2) (R(phi_in) x I) BS(pi/4,pi/2) (R(phi_ex) x I)
    (reference ``strawberryfields/ops.py:1951-2003``; fock builder ops.py:332).

    Each factor conserves total photon number, so the product is formed on the
    cutoff-(2D-1) tensors (complete photon-number blocks) and then truncated,
    which gives the exact matrix elements of the operator.
    """
    De = 2 * D - 1
    B = beamsplitter(np.pi / 4, np.pi / 2, De)
    idx = np.arange(De)
    Rin = np.exp(1j * phi_in * idx)
    Rex = np.exp(1j * phi_ex * idx)
    # (R1 X)[m,n,p,q] = e^{i a m} X ; (X R1)[m,n,p,q] = X e^{i a n}
    M = B * Rex[None, :, None, None]
    M = Rin[:, None, None, None] * M
    M = _compose2(B, M)
    return np.ascontiguousarray(M[:D, :D, :D, :D])


def cross_kerr(kappa, D):
    """CK(kappa) = exp(i kappa n1 n2) as ``mat[m,n,p,q]`` (reference ops.py:284)."""
    n = np.arange(D)
    ph = np.exp(1j * kappa * np.outer(n, n))  # [n1, n2]
    M = np.zeros((D, D, D, D), dtype=CDT)
    for i in range(D):
        for j in range(D):
            M[i, i, j, j] = ph[i, j]
    return M


# ---------------------------------------------------------------------------
# loss channel
# ---------------------------------------------------------------------------

def loss_kraus(T, D):
    """Kraus operators E_l = ((1-T)/T)^{l/2} a^l/sqrt(l!) T^{n/2} (reference ops.py:471-490)."""
    a = np.diag(np.sqrt(np.arange(1, D, dtype=np.float64)), 1).astype(CDT)
    if T == 0:
        out = []
        for i in range(D):
            P = np.zeros((D, D), dtype=CDT)
            P[0, i] = 1.0
            out.append(P)
        return out
    TT = np.diag(T ** (np.arange(D) / 2.0)).astype(CDT)
    return [((1 - T) / T) ** (l / 2.0) * (np.linalg.matrix_power(a, l) / math.sqrt(math.factorial(l))) @ TT
            for l in range(D)]


def loss_coeffs(T, D):
    """Closed-form loss superoperator coefficients ``c[n, m, l]`` such that
    ``N(T){|n><m|} = sum_l c[n,m,l] |n-l><m-l|``
    (``c = (1-T)^l T^{(n+m)/2 - l} / l! sqrt(n! m! / ((n-l)! (m-l)!))``,
    reference ``strawberryfields/ops.py:1369-1376`` and ``tfbackend/ops.py:288-315``)."""
    c = np.zeros((D, D, D), dtype=np.float64)
    for n in range(D):
        for m in range(D):
            for l in range(min(n, m) + 1):
                c[n, m, l] = ((1 - T) ** l * T ** ((n + m) / 2.0 - l) / math.factorial(l)
                              * math.sqrt(math.factorial(n) * math.factorial(m)
                                          / (math.factorial(n - l) * math.factorial(m - l))))
    return c


# ---------------------------------------------------------------------------
# state preparation and state updates
# ---------------------------------------------------------------------------

def vacuum(n, D, pure=True):
    """Vacuum state (reference ops.py:363-383)."""
    shape = [D] * (n if pure else 2 * n)
    s = np.zeros(shape, dtype=CDT)
    s.flat[0] = 1.0
    return s


def coherent_state(r, phi, D):
    """Coherent state amplitudes (reference ops.py:391-402)."""
    alpha = r * np.exp(1j * phi)
    k = np.arange(D)
    fac = np.array([math.factorial(int(i)) for i in k], dtype=np.float64)
    return np.exp(-0.5 * r * r) * alpha**k / np.sqrt(fac)


def mix(psi, n):
    """|psi><psi| with interleaved axes (reference ops.py:110-120)."""
    D = psi.shape[0]
    rho = np.multiply.outer(psi, psi.conj())  # [k0..kn-1, b0..bn-1]
    perm = []
    for i in range(n):
        perm += [i, n + i]
    return np.transpose(rho, perm).reshape([D] * (2 * n))


def _apply_axis(state, U, axis):
    """out[..., a, ...] = sum_b U[a,b] state[..., b, ...] on one axis."""
    out = np.tensordot(U, state, axes=([1], [axis]))
    return np.moveaxis(out, 0, axis)


def apply_gate1(state, U, mode, pure=True):
    """Single-mode gate (reference circuit.py:118-217): pure ``U psi`` on axis
    ``mode``; mixed ``U rho U^dag`` on the axis pair (2 mode, 2 mode + 1)."""
    if pure:
        return _apply_axis(state, U, mode)
    out = _apply_axis(state, U, 2 * mode)
    return _apply_axis(out, U.conj(), 2 * mode + 1)


def _apply_pair(state, G, ax1, ax2):
    """out[.., m, .., p, ..] = sum_{n,q} G[m,n,p,q] state[.., n, .., q, ..]."""
    out = np.tensordot(G, state, axes=([1, 3], [ax1, ax2]))  # [m, p, rest...]
    return np.moveaxis(out, [0, 1], [ax1, ax2])


def apply_gate2(state, G, mode1, mode2, pure=True):
    """Two-mode gate with ``G[out1,in1,out2,in2]`` (reference circuit.py:219-365
    for BS/MZ/S2 and the dense path of ``apply_gate_BLAS`` for cross-Kerr).
    Mixed states get ``G`` on the ket axes and ``conj(G)`` on the bra axes."""
    if pure:
        return _apply_pair(state, G, mode1, mode2)
    out = _apply_pair(state, G, 2 * mode1, 2 * mode2)
    return _apply_pair(out, G.conj(), 2 * mode1 + 1, 2 * mode2 + 1)


def apply_loss(state, T, mode, n, pure):
    """Loss channel as the Kraus sum of ``circuit.py:65-87`` (``ops.lossChannel``);
    a pure input is mixed first.  Returns the mixed output."""
    rho = mix(state, n) if pure else state
    out = np.zeros_like(rho)
    for E in loss_kraus(T, state.shape[0]):
        out += apply_gate1(rho, E, mode, pure=False)
    return out


# ---------------------------------------------------------------------------
# readouts
# ---------------------------------------------------------------------------

def all_fock_probs(state, n, pure=True):
    """|psi|^2 or diag(rho) (reference states.py:580-610)."""
    if pure:
        return (state * state.conj()).real
    D = state.shape[0]
    idx = np.arange(D)
    # diagonal over each (ket, bra) pair
    d = state
    for i in range(n):
        d = np.diagonal(d, axis1=i, axis2=i + 1)  # moves the diagonal to the end
        d = np.moveaxis(d, -1, i)
    del idx
    return d.real.copy()


def marginal(state, n, mode, pure=True):
    """Photon-number distribution of one mode (diagonal of the reduced dm of
    reference states.py:613-642, without forming the full density matrix)."""
    p = all_fock_probs(state, n, pure)
    axes = tuple(i for i in range(n) if i != mode)
    return p.sum(axis=axes)


def mean_photon(state, n, mode, pure=True):
    """(<n>, Var n) of one mode (reference states.py:657-663)."""
    p = marginal(state, n, mode, pure)
    k = np.arange(p.shape[0])
    mean = float(np.sum(k * p))
    var = float(np.sum(k * k * p) - mean * mean)
    return mean, var


def reduced_dm(state, n, mode, pure=True):
    """Single-mode reduced density matrix (reference states.py:613-642)."""
    if pure:
        x = np.moveaxis(state, mode, 0).reshape(state.shape[0], -1)
        return x @ x.conj().T
    rho = state
    D = state.shape[0]
    # trace all other modes
    keep = None
    for i in reversed(range(n)):
        if i == mode:
            continue
        rho = np.trace(rho, axis1=2 * i, axis2=2 * i + 1)
    keep = rho.reshape(D, D)
    return keep


# ---------------------------------------------------------------------------
# gate lists: forward and tape adjoint (gradient checker for the GPU sweep)
# ---------------------------------------------------------------------------
# gate kinds (same codes as the C ABI)
ROTATION, KERR, DISPLACEMENT, SQUEEZE, BEAMSPLITTER, TWO_MODE_SQUEEZE, MZGATE, CROSS_KERR = 1, 2, 3, 4, 5, 6, 7, 8
LOSS = 9


def gate_matrix(kind, p, D):
    """(matrix, [d matrix / d p_k]) of one gate in SF order.  Single-mode
    kinds give D x D matrices, two-mode kinds [out1, in1, out2, in2]."""
    n = np.arange(D)
    if kind == ROTATION:
        U = np.diag(np.exp(1j * p[0] * n)).astype(CDT)
        return U, [U * (1j * n)[None, :]]
    if kind == KERR:
        U = np.diag(np.exp(1j * p[0] * n**2)).astype(CDT)
        return U, [U * (1j * n**2)[None, :]]
    if kind == DISPLACEMENT:
        U = displacement(p[0], p[1], D)
        return U, list(grad_displacement(p[0], p[1], D))
    if kind == SQUEEZE:
        U = squeezing(p[0], p[1], D)
        return U, list(grad_squeezing(p[0], p[1], D))
    if kind == BEAMSPLITTER:
        U = beamsplitter(p[0], p[1], D)
        return U, list(grad_beamsplitter(p[0], p[1], D))
    if kind == TWO_MODE_SQUEEZE:
        U = two_mode_squeeze(p[0], p[1], D)
        return U, list(grad_two_mode_squeeze(p[0], p[1], D))
    if kind == MZGATE:
        U = mzgate(p[0], p[1], D)
        h = 1e-5
        d0 = (mzgate(p[0] + h, p[1], D) - mzgate(p[0] - h, p[1], D)) / (2 * h)
        d1 = U * (1j * n)[None, :, None, None]  # R(phi_ex) on mode 1 acts first
        return U, [d0, d1]
    if kind == CROSS_KERR:
        U = cross_kerr(p[0], D)
        nn = np.multiply.outer(n, n)  # [n1, n2]
        w = np.zeros((D, D, D, D))
        for i in range(D):
            for j in range(D):
                w[i, i, j, j] = nn[i, j]
        return U, [U * 1j * w]
    raise ValueError(f"unknown gate kind {kind}")


NPARAMS = {ROTATION: 1, KERR: 1, DISPLACEMENT: 2, SQUEEZE: 2, BEAMSPLITTER: 2, TWO_MODE_SQUEEZE: 2,
           MZGATE: 2, CROSS_KERR: 1, LOSS: 1}


def run_gates(gates, params, N, D, state=None):
    """Apply a gate list ``(kind, mode1, mode2, pidx)`` to a pure state
    (vacuum by default); returns the list of states [psi_0, ..., psi_G]."""
    psi = vacuum(N, D) if state is None else np.array(state, dtype=CDT)
    out = [psi]
    for kind, m1, m2, pi in gates:
        p = [params[pi + k] for k in range(NPARAMS[kind])]
        U, _ = gate_matrix(kind, p, D)
        if U.ndim == 2:
            psi = apply_gate1(psi, U, m1)
        else:
            psi = apply_gate2(psi, U, m1, m2)
        out.append(psi)
    return out


def homodyne_pdf(rho, phi, hbar=2.0, q_max=10.0, num_bins=100000):
    """Binned distribution of the quadrature x cos(phi) + p sin(phi) of a
    single-mode density matrix ``rho`` (reference fockbackend/circuit.py
    :724-755): rho rotated by R(-phi), physicists' Hermite polynomials by
    their recurrence, pdf times the bin width.  Returns (grid, probabilities)."""
    D = rho.shape[0]
    mw = 1.0 / hbar
    n = np.arange(D)
    U = np.diag(np.exp(-1j * phi * n))
    r = U @ rho @ U.conj().T
    q = np.linspace(-q_max, q_max, num_bins)
    x = np.sqrt(mw) * q
    H = [np.ones_like(x), 2 * x]
    for k in range(2, D):
        H.append(2 * x * H[k - 1] - 2 * (k - 1) * H[k - 2])
    dist = np.zeros(num_bins, dtype=CDT)
    for a in range(D):
        for b in range(D):
            dist += r[a, b] * H[a] * H[b] / math.sqrt(2 ** a * math.factorial(a) * 2 ** b * math.factorial(b))
    return q, (dist * np.sqrt(mw / np.pi) * np.exp(-mw * q ** 2) * (q[1] - q[0])).real


def wigner(rho, xvec, pvec, hbar=2.0):
    """Wigner function of a single-mode density matrix on the grid
    meshgrid(xvec, pvec) (shape [len(pvec), len(xvec)]): the reference's
    iterative evaluation (strawberryfields/backends/states.py:730-785).
    Grids G[n] for |m><n| are filled row by row, m = 0 first:
    G[n] = 2 A G[n-1] / sqrt(n) on row 0, then on row m the diagonal entry
    (2 conj(A) G[m] - sqrt(m) G[m-1]) / sqrt(m) and the entries right of it
    (2 A G[n-1] - sqrt(m) G_prev[n]) / sqrt(n), G_prev being row m-1; W sums
    Re rho[m][m] G[m] + 2 Re rho[m][n] G[n] (n > m) and is divided by hbar."""
    D = rho.shape[0]
    Q, P = np.meshgrid(np.asarray(xvec, dtype=float), np.asarray(pvec, dtype=float))
    A = (Q + 1j * P) / (2 * np.sqrt(hbar / 2))
    G = [np.exp(-2.0 * np.abs(A) ** 2) / np.pi + 0j]
    W = np.real(rho[0, 0]) * np.real(G[0])
    for n in range(1, D):
        G.append(2.0 * A * G[n - 1] / np.sqrt(n))
        W = W + 2 * np.real(rho[0, n] * G[n])
    for m in range(1, D):
        prev_m = G[m].copy()
        G[m] = (2 * np.conj(A) * prev_m - np.sqrt(m) * G[m - 1]) / np.sqrt(m)
        W = W + np.real(rho[m, m] * G[m])
        prev = prev_m
        for n in range(m + 1, D):
            new = (2 * A * G[n - 1] - np.sqrt(m) * prev) / np.sqrt(n)
            prev = G[n].copy()
            G[n] = new
            W = W + 2 * np.real(rho[m, n] * G[n])
    return W / hbar


def _choi(S, d):
    """choi_trick of tfbackend/ops.py:457-525: S on m modes of a Choi state
    (two-mode squeezing arcsinh 1 per mode), Husimi covariance -> Hermite
    matrix, R from its 2m x 2m corner rescaled by 1/tanh(arcsinh 1)
    on the reference half, y and C from alpha = (d_x + i d_p) / 2."""
    S = np.asarray(S, dtype=CDT)
    d = np.asarray(d, dtype=CDT)
    m = S.shape[0] // 2
    alpha = (d[:m] + 1j * d[m:]) / 2
    r = np.arcsinh(1.0)
    O, Id = np.zeros((m, m)), np.eye(m)
    choi_s = np.block([[np.cosh(r) * Id, np.sinh(r) * Id, O, O], [np.sinh(r) * Id, np.cosh(r) * Id, O, O],
                       [O, O, np.cosh(r) * Id, -np.sinh(r) * Id], [O, O, -np.sinh(r) * Id, np.cosh(r) * Id]])
    full = np.block([[S[:m, :m], O, S[:m, m:], O], [O, Id, O, O], [S[m:, :m], O, S[m:, m:], O], [O, O, O, Id]])
    Sx = full @ choi_s
    V = 0.5 * Sx @ Sx.T
    I2 = np.eye(2 * m)
    T = np.sqrt(0.5) * np.block([[I2, 1j * I2], [I2, -1j * I2]])
    sq = T @ V @ T.conj().T + 0.5 * np.eye(4 * m)
    X = np.block([[np.zeros((2 * m, 2 * m)), I2], [I2, np.zeros((2 * m, 2 * m))]])
    A = X @ (np.eye(4 * m) - np.linalg.inv(sq))
    E = np.diag(np.r_[np.ones(m), np.ones(m) / np.tanh(r)])
    R = -np.conj(E @ A[:2 * m, :2 * m] @ E)
    y = np.r_[R[:m, :m] @ alpha.conj() + alpha, R[m:, :m] @ alpha.conj()]
    at = np.r_[alpha, np.zeros(m)]
    C = np.sqrt(np.sqrt(np.linalg.det(np.eye(m) - R[:m, :m] @ R[:m, :m].conj()) + 0j)) * np.exp(
        -0.5 * np.sum(at.conj() * (at + R @ at.conj())))
    return R, y, C


def gaussian_gate_matrix(S, d, D):
    """Fock matrix of the m-mode Gaussian unitary with symplectic S (xxpp)
    and displacement d, as the reference's TF backend forms it
    (strawberryfields/backends/tfbackend/ops.py:457-572): choi_trick's
    (R, y, C), then the renormalised multidimensional Hermite tensor of the
    third-party thewalrus (not vendored; restated from its recurrence
    G[k] = (y_i G[k-e_i] - sum_j R_ij sqrt(k_j - d_ij) G[k-e_i-e_j]) / sqrt(k_i),
    i the first nonzero index, G[0] = C).  Returns [out_1..out_m, in_1..in_m].
    Pinned by tests/test_oracle.py against the exact truncated matrices of
    the squeezer, displacement, rotation, beamsplitter and two-mode squeezer."""
    import itertools

    R, y, C = _choi(S, d)
    n = len(y)
    G = np.zeros((D,) * n, dtype=CDT)
    for k in itertools.product(range(D), repeat=n):
        if not any(k):
            G[k] = C
            continue
        i = next(j for j in range(n) if k[j] > 0)
        km = list(k)
        km[i] -= 1
        v = y[i] * G[tuple(km)]
        for j in range(n):
            if km[j] > 0:
                kk = list(km)
                kk[j] -= 1
                v -= R[i, j] * math.sqrt(km[j]) * G[tuple(kk)]
        G[k] = v / math.sqrt(k[i])
    return G


def apply_gate_modes(state, G, modes, pure=True):
    """Apply G [out_1..out_k, in_1..in_k] to ``modes`` of a ket, or as
    G rho G^dagger to a density matrix (interleaved axes)."""
    k = len(modes)
    axes_k = list(modes) if pure else [2 * m for m in modes]
    out = np.tensordot(G, state, axes=(list(range(k, 2 * k)), axes_k))
    out = np.moveaxis(out, list(range(k)), axes_k)
    if pure:
        return out
    axes_b = [2 * m + 1 for m in modes]
    out = np.tensordot(G.conj(), out, axes=(list(range(k, 2 * k)), axes_b))
    return np.moveaxis(out, list(range(k)), axes_b)


def homodyne_project(state, phi, x, mode, n, pure=True, hbar=2.0):
    """State after a homodyne outcome ``x`` on ``mode`` (reference
    circuit.py:766-795): |0><x_phi| applied to the mode, with x_phi =
    R(phi) D(alpha) times the truncated infinitely squeezed vacuum, alpha =
    x sqrt(1 / (2 hbar)); renormalised (2-norm for a ket, trace for a
    density matrix)."""
    D = state.shape[0]
    sq = np.array([(-0.5) ** (k // 2) * math.sqrt(math.factorial(k)) / math.factorial(k // 2) if k % 2 == 0 else 0.0
                   for k in range(D)], dtype=CDT)
    alpha = x * math.sqrt(1.0 / (2 * hbar))
    eig = phase(phi, D) @ displacement(abs(alpha), np.angle(alpha), D) @ sq
    P = np.zeros((D, D), dtype=CDT)
    P[0, :] = eig.conj()
    out = apply_gate1(state, P, mode, pure)
    if pure:
        return out / np.linalg.norm(out)
    tr = np.real(np.trace(out.reshape(D ** n, D ** n) if n == 1 else
                          np.transpose(out, [2 * i for i in range(n)] + [2 * i + 1 for i in range(n)])
                          .reshape(D ** n, D ** n)))
    return out / tr


def run_gates_mixed(gates, params, N, D, rho=None):
    """Density-matrix run of a gate list (vacuum by default): unitaries as
    ``U rho U^dag`` (reference circuit.py:186-217), ``LOSS`` (parameter T) as
    the Kraus sum of circuit.py:65-87.  Returns the final rho."""
    rho = vacuum(N, D, pure=False) if rho is None else np.array(rho, dtype=CDT)
    for kind, m1, m2, pi in gates:
        p = [params[pi + k] for k in range(NPARAMS[kind])]
        if kind == LOSS:
            rho = apply_loss(rho, p[0], m1, N, pure=False)
            continue
        U, _ = gate_matrix(kind, p, D)
        rho = apply_gate1(rho, U, m1, pure=False) if U.ndim == 2 else apply_gate2(rho, U, m1, m2, pure=False)
    return rho


def adjoint_grads(gates, params, N, D, grad_final, state=None):
    """Reverse sweep over the stored tape.  ``grad_final`` is dL/dpsi of the
    final state in the convention dL/dRe + i dL/dIm; returns dL/dparams.
    Per gate: dL/dp = Re sum_{ab} C[a,b] dU[a,b]/dp with
    C = sum_rest conj(lam_out[a]) psi_in[b], and lam_in = U^dagger lam_out."""
    states = run_gates(gates, params, N, D, state)
    g = np.zeros(len(params))
    lam = np.array(grad_final, dtype=CDT)
    for k in range(len(gates) - 1, -1, -1):
        kind, m1, m2, pi = gates[k]
        p = [params[pi + j] for j in range(NPARAMS[kind])]
        U, dUs = gate_matrix(kind, p, D)
        psi_in = states[k]
        if U.ndim == 2:
            lo = np.moveaxis(lam, m1, 0).reshape(D, -1)
            pi_ = np.moveaxis(psi_in, m1, 0).reshape(D, -1)
            C = lo.conj() @ pi_.T
            for j, dU in enumerate(dUs):
                g[pi + j] += float(np.real(np.sum(C * dU)))
            lam = apply_gate1(lam, U.conj().T, m1)
        else:
            lo = np.moveaxis(lam, [m1, m2], [0, 1]).reshape(D, D, -1)
            pi_ = np.moveaxis(psi_in, [m1, m2], [0, 1]).reshape(D, D, -1)
            # C[m,n,p,q] = sum_r conj(lo[m,p,r]) pi[n,q,r], as one GEMM
            C = (lo.conj().reshape(D * D, -1) @ pi_.reshape(D * D, -1).T).reshape(D, D, D, D).transpose(0, 2, 1, 3)
            for j, dU in enumerate(dUs):
                g[pi + j] += float(np.real(np.sum(C * dU)))
            Uh = np.conj(U).transpose(1, 0, 3, 2)  # [in1, out1, in2, out2] -> acts as U^dagger
            lam = apply_gate2(lam, Uh, m1, m2)
    return g
