"""Compiled density-matrix circuits (pure=False): forward sweeps against the
reference Circuit's golden vectors and the oracle; adjoint gradients (gate
parameters and loss transmissivities) against central differences of the
oracle, the complex128 result and the checkpointed sweep.

Tolerances: 1e-12 (complex128) / 1e-5 (complex64) on states; FP64 gradients
to 1e-6 relative against central differences with h = 1e-6; complex64
gradients to 1e-4 relative against complex128.
"""
import os

import numpy as np
import pytest
import torch

from oracle import fock_oracle as fo
from tests.gatelist import ops_to_gates
from tests.golden.make_golden import decode

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

def _gate_case(f):
    z = np.load(os.path.join(GOLDEN, f))
    return not z["pure"] and not np.any(z["ops"][:, 0] == 10)  # no measurements


MIXED = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz") and _gate_case(f))


def _circuit(N, D, gates, npar, dtype, **kw):
    from strawberryfields_gb300 import CompiledCircuit

    return CompiledCircuit(N, D, gates, npar, dtype=dtype, pure=False, **kw)


@pytest.mark.parametrize("dtype,tol", [(torch.complex128, 1e-12), (torch.complex64, 1e-5)])
@pytest.mark.parametrize("case", MIXED)
def test_mixed_plan_reproduces_golden(cuda, case, dtype, tol):
    z = np.load(os.path.join(GOLDEN, case + ".npz"))
    gates, params = ops_to_gates(decode(z["ops"]))
    circ = _circuit(int(z["N"]), int(z["D"]), gates, len(params), dtype)
    rho = circ(torch.tensor(params, device=cuda, dtype=torch.float64)).detach().cpu().numpy().astype(np.complex128)
    assert np.abs(rho - z["state"]).max() < tol


def _random_mixed(N, seed):
    """Every gate kind, swapped pairs, and a loss channel on each mode."""
    rng = np.random.default_rng(seed)
    gates, params = [], []

    def add(kind, m1, m2, *p):
        gates.append((kind, m1, m2, len(params)))
        params.extend(p)

    for m in range(N):
        add(4, m, -1, rng.uniform(0, 0.4), rng.uniform(0, 6.28))
        add(3, m, -1, rng.uniform(0, 0.4), rng.uniform(0, 6.28))
    add(5, 0, 1, rng.uniform(0, 1.5), rng.uniform(0, 6.28))
    add(1, 0, -1, rng.uniform(0, 6.28))
    add(2, 1, -1, rng.uniform(0, 0.1))
    add(9, 1, -1, rng.uniform(0.7, 1.0))
    add(6, N - 1, 0, rng.uniform(0, 0.3), rng.uniform(0, 6.28))
    add(8, 0, N - 1, rng.uniform(0, 0.1))
    add(7, 1, 0, rng.uniform(0, 6.28), rng.uniform(0, 6.28))
    for m in range(N):
        add(9, m, -1, rng.uniform(0.7, 1.0))
    add(2, 0, -1, rng.uniform(0, 0.1))
    add(1, N - 1, -1, rng.uniform(0, 6.28))
    return gates, np.array(params)


def test_mixed_plan_matches_oracle(cuda):
    N, D = 3, 5
    gates, params = _random_mixed(N, 11)
    ref = fo.run_gates_mixed(gates, params, N, D)
    for dtype, tol in ((torch.complex128, 1e-12), (torch.complex64, 1e-5)):
        rho = _circuit(N, D, gates, len(params), dtype)(torch.tensor(params, device=cuda, dtype=torch.float64))
        assert np.abs(rho.detach().cpu().numpy().astype(np.complex128) - ref).max() < tol


def _weights(N, D, seed):
    return np.random.default_rng(seed).uniform(-1, 1, size=(D,) * N)


def _torch_loss(rho, w, N):
    """L = sum_n w[n] <n|rho|n> (photon-number statistics of all modes)."""
    D = rho.shape[0]
    perm = [2 * i for i in range(N)] + [2 * i + 1 for i in range(N)]
    diag = torch.diagonal(rho.permute(perm).reshape(D ** N, D ** N)).real.reshape([D] * N)
    return torch.sum(torch.as_tensor(w, device=rho.device, dtype=diag.dtype) * diag)


def _np_loss(rho, w, N):
    D = rho.shape[0]
    perm = [2 * i for i in range(N)] + [2 * i + 1 for i in range(N)]
    diag = np.diagonal(np.transpose(rho, perm).reshape(D ** N, D ** N)).real.reshape([D] * N)
    return float(np.sum(w * diag))


def _grad(circ, params, w, N, cuda):
    p = torch.tensor(params, device=cuda, dtype=torch.float64, requires_grad=True)
    loss = _torch_loss(circ(p), w, N)
    loss.backward()
    return p.grad.detach().cpu().numpy(), float(loss)


def test_mixed_gradient_matches_central_differences(cuda):
    N, D = 2, 5
    gates, params = _random_mixed(N, 5)
    w = _weights(N, D, 1)
    g, _ = _grad(_circuit(N, D, gates, len(params), torch.complex128), params, w, N, cuda)
    h = 1e-6
    fd = np.zeros(len(params))
    for i in range(len(params)):
        pp, pm = params.copy(), params.copy()
        pp[i] += h
        pm[i] -= h
        fd[i] = (_np_loss(fo.run_gates_mixed(gates, pp, N, D), w, N) -
                 _np_loss(fo.run_gates_mixed(gates, pm, N, D), w, N)) / (2 * h)
    assert np.linalg.norm(g - fd) <= 1e-6 * np.linalg.norm(fd)
    # the loss transmissivities reach the photon statistics
    t_idx = [pi for kind, _, _, pi in gates if kind == 9]
    assert np.all(np.abs(fd[t_idx]) > 1e-9)


def test_mixed_gradient_c64_and_checkpoints(cuda):
    N, D = 3, 6
    gates, params = _random_mixed(N, 8)
    w = _weights(N, D, 2)
    g128, _ = _grad(_circuit(N, D, gates, len(params), torch.complex128), params, w, N, cuda)
    g64, _ = _grad(_circuit(N, D, gates, len(params), torch.complex64), params, w, N, cuda)
    assert np.linalg.norm(g64 - g128) <= 1e-4 * np.linalg.norm(g128)
    gk, _ = _grad(_circuit(N, D, gates, len(params), torch.complex128, checkpoint=3), params, w, N, cuda)
    assert np.linalg.norm(gk - g128) <= 1e-12 * np.linalg.norm(g128)


@pytest.mark.parametrize("k,slots", [(1000, 3), (1000, 4), (1000, 7), (9, 3), (9, 5), (9, 8)])
def test_recursive_recompute_matches_stored_states(cuda, k, slots):
    """A checkpoint segment recomputed recursively in `slots` states gives the
    same gradient as keeping every state (same kernels on the same inputs)."""
    N, D = 3, 5
    gates, params = _random_mixed(N, 4)
    w = _weights(N, D, 3)
    g1, l1 = _grad(_circuit(N, D, gates, len(params), torch.complex128), params, w, N, cuda)
    gk, lk = _grad(_circuit(N, D, gates, len(params), torch.complex128, checkpoint=k, recompute_slots=slots),
                   params, w, N, cuda)
    assert lk == l1
    np.testing.assert_allclose(gk, g1, rtol=1e-13, atol=1e-15)


def test_recursive_recompute_pure_qnn(cuda):
    from strawberryfields_gb300 import CompiledCircuit
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params

    gates, npar = qnn_gates(3, 3)
    params = qnn_params(gates, npar, seed=2)
    t = torch.randn(7, 7, 7, dtype=torch.complex64, device=cuda)

    def grad(circ):
        p = torch.tensor(params, device=cuda, requires_grad=True)
        psi = circ(p)
        loss = torch.abs(torch.sum(t.conj() * psi)) ** 2
        loss.backward()
        return p.grad.detach().cpu().numpy()

    g1 = grad(CompiledCircuit(3, 7, gates, npar, dtype=torch.complex64, device=cuda))
    g2 = grad(CompiledCircuit(3, 7, gates, npar, dtype=torch.complex64, device=cuda, checkpoint=20, recompute_slots=4))
    np.testing.assert_allclose(g2, g1, rtol=1e-6, atol=1e-9)
