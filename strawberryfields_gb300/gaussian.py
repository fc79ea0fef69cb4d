"""Host side of the general N-mode Gaussian gate (``Ggate``).

The reference applies ``Ggate(S, d)`` only in its TF backend
(``strawberryfields/backends/tfbackend/ops.py:457-572``, called from
``tfbackend/circuit.py:565``): ``choi_trick`` turns the symplectic matrix S
(xxpp ordering) and the displacement d into the parameters (R, y, C) of a
renormalised multidimensional Hermite tensor -- the Fock matrix of the gate --
which ``fock_gaussian_gate_matrix`` evaluates on the device in FP64.  The
steps below are that map: S acts on m modes of a two-mode-squeezed
Choi state of squeezing arcsinh(1) (the Fock-space Choi isomorphism), the
Gaussian state's Husimi covariance gives the Hermite matrix
A = X (I - sigma_Q^{-1}), and R = -conj(E A_11 E) with E rescaling the
reference half by 1/tanh(arcsinh 1); y and C follow from the displacement
alpha = (d_x + i d_p) / 2.
"""

import numpy as np


def is_symplectic(S, rtol=1e-05, atol=1e-06):
    """S^T Omega S == Omega in xxpp ordering."""
    S = np.asarray(S)
    n2 = S.shape[0]
    if S.ndim != 2 or S.shape[1] != n2 or n2 % 2:
        return False
    m = n2 // 2
    Om = np.block([[np.zeros((m, m)), np.eye(m)], [-np.eye(m), np.zeros((m, m))]])
    return bool(np.allclose(S.T @ Om @ S, Om, rtol=rtol, atol=atol))


def choi_parameters(S, d):
    """(R [2m, 2m], y [2m], C) of the Gaussian unitary with symplectic S and
    displacement d (tfbackend/ops.py:457-525)."""
    S = np.asarray(S, dtype=np.complex128)
    d = np.asarray(d, dtype=np.complex128)
    m = S.shape[0] // 2
    alpha = (d[:m] + 1j * d[m:]) / 2
    r0 = np.arcsinh(1.0)
    Z = np.zeros((m, m))
    I = np.eye(m)
    ch, sh = np.cosh(r0) * I, np.sinh(r0) * I
    tmsv = np.block([[ch, sh, Z, Z], [sh, ch, Z, Z], [Z, Z, ch, -sh], [Z, Z, -sh, ch]])
    s_ext = np.block([[S[:m, :m], Z, S[:m, m:], Z], [Z, I, Z, Z], [S[m:, :m], Z, S[m:, m:], Z], [Z, Z, Z, I]])
    s_ext = s_ext @ tmsv
    cov = 0.5 * s_ext @ s_ext.T
    I2 = np.eye(2 * m)
    W = np.sqrt(0.5) * np.block([[I2, 1j * I2], [I2, -1j * I2]])
    sigma_q = W @ cov @ W.conj().T + 0.5 * np.eye(4 * m)
    Z2 = np.zeros((2 * m, 2 * m))
    A = np.block([[Z2, I2], [I2, Z2]]) @ (np.eye(4 * m) - np.linalg.inv(sigma_q))
    E = np.diag(np.concatenate([np.ones(m), np.ones(m) / np.tanh(r0)]))
    R = -np.conj(E @ A[: 2 * m, : 2 * m] @ E)
    y = np.concatenate([R[:m, :m] @ np.conj(alpha) + alpha, R[m:, :m] @ np.conj(alpha)])
    a_ext = np.concatenate([alpha, np.zeros(m)])
    zeta = a_ext + R @ np.conj(a_ext)
    C = np.sqrt(np.sqrt(np.linalg.det(np.eye(m) - R[:m, :m] @ np.conj(R[:m, :m])) + 0j)) * np.exp(
        -0.5 * np.sum(np.conj(a_ext) * zeta))
    return R, y, complex(C)


def check_gate(S, d):
    """The reference's argument checks (tfbackend/ops.py:1115-1131)."""
    S = np.asarray(S)
    d = np.asarray(d)
    if S.shape[0] != d.shape[0]:
        raise ValueError("The matrix S and the vector d do not have compatible dimensions")
    if not is_symplectic(S.real if np.iscomplexobj(S) else S):
        raise ValueError("The matrix S is not symplectic")
