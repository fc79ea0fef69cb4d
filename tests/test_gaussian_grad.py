"""Gradients of the Gaussian gate (strawberryfields_gb300/gaussian.py):
the torch restatement of the Choi parameters against the numpy one, and the
Hermite-tensor backward (dG/dy, dG/dR, dG/dC identities) chained through it
against central differences of the oracle's gate matrix in S and d -- on the
CPU, with the oracle's matrix standing in for the device build.  The device
path (build + apply + their backward) is checked in
tests/test_gpu_gaussian_grad.py."""
import numpy as np
import pytest
import torch

from oracle import fock_oracle as fo


def _gate(m, seed):
    from scipy.stats import unitary_group

    rng = np.random.default_rng(seed)
    U = unitary_group.rvs(m, random_state=seed)
    O = np.block([[U.real, -U.imag], [U.imag, U.real]])
    r = rng.uniform(0.05, 0.3, m)
    S = O @ np.diag(np.r_[np.exp(-r), np.exp(r)])
    V = unitary_group.rvs(m, random_state=seed + 7)
    S = np.block([[V.real, -V.imag], [V.imag, V.real]]) @ S
    d = rng.normal(size=2 * m) * 0.3
    return S, d


def test_choi_parameters_torch_matches_numpy():
    from strawberryfields_gb300.gaussian import choi_parameters, choi_parameters_torch

    for m in (1, 2, 3):
        S, d = _gate(m, m)
        R, y, C = choi_parameters(S, d)
        Rt, yt, Ct = choi_parameters_torch(torch.tensor(S), torch.tensor(d))
        assert np.abs(R - Rt.numpy()).max() < 1e-13
        assert np.abs(y - yt.numpy()).max() < 1e-13
        assert abs(C - complex(Ct)) < 1e-13


@pytest.mark.parametrize("m,D", [(1, 8), (2, 5)])
def test_hermite_backward_through_choi_matches_central_differences(m, D):
    from strawberryfields_gb300.gaussian import _HermiteMatrix, choi_parameters_torch

    S, d = _gate(m, 10 + m)
    rng = np.random.default_rng(3)
    g = rng.normal(size=(D,) * (2 * m)) + 1j * rng.normal(size=(D,) * (2 * m))

    class OracleHermite(torch.autograd.Function):
        @staticmethod
        def forward(ctx, R, y, C):
            G = torch.as_tensor(fo.gaussian_gate_matrix(S_now[0], d_now[0], D))
            ctx.save_for_backward(G, C.detach())
            return G

        @staticmethod
        def backward(ctx, grad):
            G, C = ctx.saved_tensors
            return _HermiteMatrix.grads(G, C, grad)

    St = torch.tensor(S, requires_grad=True)
    dt = torch.tensor(d, requires_grad=True)
    S_now, d_now = [S], [d]
    R, y, C = choi_parameters_torch(St, dt)
    G = OracleHermite.apply(R, y, C)
    loss = torch.real(torch.sum(torch.conj(torch.as_tensor(g)) * G))
    loss.backward()

    def L(S_, d_):
        return float(np.real(np.sum(np.conj(g) * fo.gaussian_gate_matrix(S_, d_, D))))

    h = 1e-6
    fd_S = np.zeros_like(S)
    for i in range(S.shape[0]):
        for j in range(S.shape[1]):
            E = np.zeros_like(S)
            E[i, j] = h
            fd_S[i, j] = (L(S + E, d) - L(S - E, d)) / (2 * h)
    fd_d = np.array([(L(S, d + h * e) - L(S, d - h * e)) / (2 * h) for e in np.eye(len(d))])
    scale = max(np.abs(fd_S).max(), np.abs(fd_d).max())
    assert np.abs(St.grad.numpy() - fd_S).max() < 1e-6 * scale
    assert np.abs(dt.grad.numpy() - fd_d).max() < 1e-6 * scale
