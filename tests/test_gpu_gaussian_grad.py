"""The differentiable Gaussian gate on the GPU (gaussian.gaussian_gate_torch:
the Fock matrix built on the device from the Choi parameters, applied by the
dense k-mode kernel, with the Hermite-tensor backward and the apply's
adjoint) against the oracle: the output state at 1e-12, and the gradients
of |<t|G psi>|^2 with respect to S, d and psi against central differences
of the oracle (the TF backend's custom gradient, tfbackend/ops.py:517-542,
gives the same derivatives)."""
import numpy as np
import pytest

from oracle import fock_oracle as fo
from tests.test_gaussian_grad import _gate

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("modes", [[1], [2, 0]])
def test_gaussian_gate_gradients_match_central_differences(cuda, modes):
    import torch
    from strawberryfields_gb300.gaussian import gaussian_gate_torch

    N, D = 3, 5
    m = len(modes)
    S, d = _gate(m, 20 + m)
    rng = np.random.default_rng(5)
    psi = rng.normal(size=(D,) * N) + 1j * rng.normal(size=(D,) * N)
    psi /= np.linalg.norm(psi)
    t = rng.normal(size=(D,) * N) + 1j * rng.normal(size=(D,) * N)
    t /= np.linalg.norm(t)

    St = torch.tensor(S, device=cuda, requires_grad=True)
    dt = torch.tensor(d, device=cuda, requires_grad=True)
    pt = torch.tensor(psi, device=cuda, requires_grad=True)
    out = gaussian_gate_torch(pt, St, dt, modes)
    ref_out = fo.apply_gate_modes(psi, fo.gaussian_gate_matrix(S, d, D), modes)
    assert np.abs(out.detach().cpu().numpy() - ref_out).max() < 1e-12
    s = torch.sum(torch.as_tensor(t, device=cuda).conj() * out)
    (s.real ** 2 + s.imag ** 2).backward()

    def L(S_, d_, psi_):
        o = fo.apply_gate_modes(psi_, fo.gaussian_gate_matrix(S_, d_, D), modes)
        return abs(np.vdot(t, o)) ** 2

    h = 1e-6
    fd_S = np.zeros_like(S)
    for i in range(S.shape[0]):
        for j in range(S.shape[1]):
            E = np.zeros_like(S)
            E[i, j] = h
            fd_S[i, j] = (L(S + E, d, psi) - L(S - E, d, psi)) / (2 * h)
    fd_d = np.array([(L(S, d + h * e, psi) - L(S, d - h * e, psi)) / (2 * h) for e in np.eye(2 * m)])
    scale = max(np.abs(fd_S).max(), np.abs(fd_d).max())
    assert np.abs(St.grad.cpu().numpy() - fd_S).max() < 1e-6 * scale
    assert np.abs(dt.grad.cpu().numpy() - fd_d).max() < 1e-6 * scale
    # dL/dpsi in the torch convention dL/dRe + i dL/dIm, at a few entries
    gp = pt.grad.cpu().numpy()
    for idx in [(0, 0, 0), (1, 2, 3), (4, 1, 0)]:
        E = np.zeros_like(psi)
        E[idx] = h
        fd = (L(S, d, psi + E) - L(S, d, psi - E)) / (2 * h) + 1j * (
            L(S, d, psi + 1j * E) - L(S, d, psi - 1j * E)) / (2 * h)
        assert abs(gp[idx] - fd) < 1e-6 * max(abs(fd), 1e-3)
