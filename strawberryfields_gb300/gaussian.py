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


# ---------------------------------------------------------------------------
# differentiable Gaussian gate (the TF backend's custom gradient,
# tfbackend/ops.py:517-542)
# ---------------------------------------------------------------------------

def choi_parameters_torch(S, d):
    """``choi_parameters`` as torch operations (complex128), differentiable in
    the symplectic matrix S (xxpp, real [2m, 2m]) and the displacement d
    (real [2m])."""
    import torch

    S = torch.as_tensor(S).to(torch.complex128)
    d = torch.as_tensor(d).to(torch.complex128)
    dev = S.device
    m = S.shape[0] // 2
    alpha = (d[:m] + 1j * d[m:]) / 2
    r0 = float(np.arcsinh(1.0))
    Z = torch.zeros((m, m), dtype=torch.complex128, device=dev)
    I = torch.eye(m, dtype=torch.complex128, device=dev)
    ch, sh = float(np.cosh(r0)) * I, float(np.sinh(r0)) * I
    tmsv = torch.cat([torch.cat([ch, sh, Z, Z], 1), torch.cat([sh, ch, Z, Z], 1),
                      torch.cat([Z, Z, ch, -sh], 1), torch.cat([Z, Z, -sh, ch], 1)], 0)
    s_ext = torch.cat([torch.cat([S[:m, :m], Z, S[:m, m:], Z], 1), torch.cat([Z, I, Z, Z], 1),
                       torch.cat([S[m:, :m], Z, S[m:, m:], Z], 1), torch.cat([Z, Z, Z, I], 1)], 0)
    s_ext = s_ext @ tmsv
    cov = 0.5 * s_ext @ s_ext.T
    I2 = torch.eye(2 * m, dtype=torch.complex128, device=dev)
    W = float(np.sqrt(0.5)) * torch.cat([torch.cat([I2, 1j * I2], 1), torch.cat([I2, -1j * I2], 1)], 0)
    sigma_q = W @ cov @ W.conj().T + 0.5 * torch.eye(4 * m, dtype=torch.complex128, device=dev)
    Z2 = torch.zeros((2 * m, 2 * m), dtype=torch.complex128, device=dev)
    X = torch.cat([torch.cat([Z2, I2], 1), torch.cat([I2, Z2], 1)], 0)
    A = X @ (torch.eye(4 * m, dtype=torch.complex128, device=dev) - torch.linalg.inv(sigma_q))
    e = torch.cat([torch.ones(m, dtype=torch.complex128, device=dev),
                   torch.full((m,), 1.0 / float(np.tanh(r0)), dtype=torch.complex128, device=dev)])
    R = -torch.conj(e[:, None] * A[: 2 * m, : 2 * m] * e[None, :])
    y = torch.cat([R[:m, :m] @ alpha.conj() + alpha, R[m:, :m] @ alpha.conj()])
    a_ext = torch.cat([alpha, torch.zeros(m, dtype=torch.complex128, device=dev)])
    zeta = a_ext + R @ a_ext.conj()
    C = torch.sqrt(torch.sqrt(torch.linalg.det(I - R[:m, :m] @ R[:m, :m].conj()))) * torch.exp(
        -0.5 * torch.sum(a_ext.conj() * zeta))
    return R, y, C


class _HermiteMatrix:
    """Autograd of the Gaussian gate's Fock matrix G[k] = C H_k(R, y) /
    sqrt(k!) in its Choi parameters.  The renormalised Hermite tensor has
    dG[k]/dy_i = sqrt(k_i) G[k - e_i], dG[k]/dR_ij = -1/2 sqrt(k_i (k_j - d_ij))
    G[k - e_i - e_j] (R as a general matrix; a symmetric change of R_ij and
    R_ji adds both) and dG/dC = G / C -- the derivatives of its generating
    function exp(x.y - x.R.x / 2).  The forward build runs on the device
    (fock_gaussian_gate_matrix); the backward contracts the incoming gradient
    with shifted copies of G (torch convention: grad_p = sum grad_G *
    conj(dG/dp))."""

    @staticmethod
    def build(R, y, C, D, device):
        import ctypes

        import torch

        from . import _lib as L

        m = y.shape[0] // 2
        Rh = np.ascontiguousarray(R.detach().cpu().numpy(), dtype=np.complex128).view(np.float64)
        yh = np.ascontiguousarray(y.detach().cpu().numpy(), dtype=np.complex128).view(np.float64)
        c = complex(C.detach().cpu())
        Ch = np.array([c.real, c.imag], dtype=np.float64)
        G = torch.empty([D] * (2 * m), dtype=torch.complex128, device=device)
        L.check(L.load().fock_gaussian_gate_matrix(m, D, Rh.ctypes.data_as(ctypes.c_void_p),
                                                   yh.ctypes.data_as(ctypes.c_void_p),
                                                   Ch.ctypes.data_as(ctypes.c_void_p), G.data_ptr(),
                                                   torch.cuda.current_stream(device).cuda_stream),
                "fock_gaussian_gate_matrix")
        return G

    @staticmethod
    def grads(G, C, g):
        """(grad_R, grad_y, grad_C) from grad_G = g."""
        import torch

        n = G.dim()
        D = G.shape[0]
        dev = G.device
        k = torch.arange(D, dtype=torch.float64, device=dev)

        def along(w, ax):
            shape = [1] * n
            shape[ax] = D
            return w.reshape(shape)

        gy = torch.zeros(n, dtype=torch.complex128, device=dev)
        gR = torch.zeros((n, n), dtype=torch.complex128, device=dev)
        for i in range(n):
            dst = [slice(None)] * n
            src = [slice(None)] * n
            dst[i], src[i] = slice(1, None), slice(0, -1)
            w = along(torch.sqrt(k), i)[tuple(dst)]
            gy[i] = torch.sum(g[tuple(dst)] * torch.conj(w * G[tuple(src)]))
            for j in range(n):
                dst = [slice(None)] * n
                src = [slice(None)] * n
                if i == j:
                    dst[i], src[i] = slice(2, None), slice(0, -2)
                    w = along(torch.sqrt(k * (k - 1).clamp_min(0)), i)[tuple(dst)]
                else:
                    dst[i], src[i] = slice(1, None), slice(0, -1)
                    dst[j], src[j] = slice(1, None), slice(0, -1)
                    w = (along(torch.sqrt(k), i) * along(torch.sqrt(k), j))[tuple(dst)]
                gR[i, j] = torch.sum(g[tuple(dst)] * torch.conj(-0.5 * w * G[tuple(src)]))
        gC = torch.sum(g * torch.conj(G / C))
        return gR, gy, gC


def _hermite_function():
    import torch

    class HermiteFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, R, y, C, D):
            G = _HermiteMatrix.build(R, y, C, D, torch.device("cuda", torch.cuda.current_device()))
            ctx.save_for_backward(G, C.detach())
            return G

        @staticmethod
        def backward(ctx, g):
            G, C = ctx.saved_tensors
            gR, gy, gC = _HermiteMatrix.grads(G, C.to(G.device), g)
            return gR, gy, gC, None

    class ApplyFn(torch.autograd.Function):
        """psi' = G psi on `modes` of a ket (complex128), through
        fock_apply_modes; backward: G^dagger lam (the same kernel with the
        conjugate-transposed matrix) and grad_G = sum_rest lam conj(psi)."""

        @staticmethod
        def forward(ctx, G, psi, modes):
            out = _apply_modes(G, psi, modes)
            ctx.save_for_backward(G, psi)
            ctx.modes = modes
            return out

        @staticmethod
        def backward(ctx, lam):
            G, psi = ctx.saved_tensors
            modes = ctx.modes
            k = len(modes)
            Dk = psi.shape[0] ** k
            Gd = G.reshape(Dk, Dk).conj().T.contiguous().reshape(G.shape)
            gpsi = _apply_modes(Gd, lam.contiguous().to(torch.complex128), modes)
            lm = torch.movedim(lam.to(torch.complex128), modes, list(range(k))).reshape(Dk, -1)
            pm = torch.movedim(psi, modes, list(range(k))).reshape(Dk, -1)
            gG = (lm @ pm.conj().T).reshape(G.shape)
            return gG, gpsi, None

    return HermiteFn, ApplyFn


def _apply_modes(G, psi, modes):
    import ctypes

    import torch

    from . import _lib as L

    lib = L.load()
    N, D, k = psi.dim(), psi.shape[0], len(modes)
    dev = psi.device
    ws = torch.empty(int(lib.fock_apply_modes_workspace_bytes(k, D, L.C128)), dtype=torch.uint8, device=dev)
    out = torch.empty_like(psi)
    md = (ctypes.c_int * k)(*modes)
    L.check(lib.fock_apply_modes(N, D, 1, L.C128, k, md, G.contiguous().data_ptr(), psi.contiguous().data_ptr(),
                                 out.data_ptr(), None, ws.data_ptr(), torch.cuda.current_stream(dev).cuda_stream),
            "fock_apply_modes")
    return out


_FNS = None


def gaussian_gate_torch(psi, S, d, modes):
    """Apply the Gaussian unitary with symplectic S (xxpp) and displacement d
    to ``modes`` of the complex128 ket ``psi`` ([D]*N on the GPU), as a
    differentiable function of psi, S and d (torch tensors).  The gradient
    with respect to S is the plain derivative of the loss, as the TF
    backend's custom gradient gives it (tfbackend/ops.py:517-542); a step
    along it leaves the symplectic group (the reference's
    update_symplectic, tfbackend/ops.py:545, maps it back)."""
    global _FNS
    import torch

    if _FNS is None:
        _FNS = _hermite_function()
    HermiteFn, ApplyFn = _FNS
    modes = [int(m) for m in modes]
    S = torch.as_tensor(S, dtype=torch.float64, device=psi.device)
    d = torch.as_tensor(d, dtype=torch.float64, device=psi.device)
    R, y, C = choi_parameters_torch(S, d)
    G = HermiteFn.apply(R, y, C, psi.shape[0])
    return ApplyFn.apply(G, psi.to(torch.complex128), modes)
