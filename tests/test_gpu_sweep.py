"""Persistent sweeps (one cooperative launch per forward / adjoint sweep)
against the per-op launches and the complex128 result.

FOCK_GB300_SWEEP_MAX_BYTES, read when a plan is created, turns the persistent
sweeps on (a byte limit) or off (0, the default).  Forward states agree
exactly (same per-column arithmetic); the gradients differ only in the order
of the FP32 partial sums.
"""

import numpy as np
import pytest
import torch

from strawberryfields_gb300 import CompiledCircuit
from strawberryfields_gb300.qnn import qnn_gates, qnn_params, target_state

pytestmark = pytest.mark.gpu


@pytest.fixture
def persistent(monkeypatch):
    monkeypatch.setenv("FOCK_GB300_SWEEP_MAX_BYTES", str(1 << 30))


def _loss_grad(circ, p, t):
    p = p.detach().clone().requires_grad_(True)
    psi = circ(p)
    s = torch.sum(t.to(psi.dtype).conj() * psi)
    loss = 1 - (s.real ** 2 + s.imag ** 2)
    loss.backward()
    return psi.detach(), p.grad.detach(), float(loss)


@pytest.mark.parametrize("modes,cutoff,layers", [(3, 6, 2), (4, 8, 1), (2, 12, 3), (5, 5, 1)])
def test_persistent_matches_per_op(cuda, persistent, monkeypatch, modes, cutoff, layers):
    gates, npar = qnn_gates(modes, layers)
    params = torch.tensor(qnn_params(gates, npar, seed=3), device=cuda)
    t = torch.as_tensor(target_state(modes, cutoff, 4, 7), device=cuda)
    circ = CompiledCircuit(modes, cutoff, gates, npar, dtype=torch.complex64, device=cuda)
    psi_p, g_p, l_p = _loss_grad(circ, params, t)
    pers, err = circ.sweep_status()
    assert pers and err == 0
    monkeypatch.setenv("FOCK_GB300_SWEEP_MAX_BYTES", "0")
    ref = CompiledCircuit(modes, cutoff, gates, npar, dtype=torch.complex64, device=cuda)
    assert not ref.sweep_status()[0]
    psi_r, g_r, l_r = _loss_grad(ref, params, t)
    assert torch.equal(psi_p, psi_r)
    gscale = float(torch.linalg.vector_norm(g_r))
    assert float(torch.linalg.vector_norm(g_p - g_r)) <= 1e-5 * gscale
    # both against complex128
    c128 = CompiledCircuit(modes, cutoff, gates, npar, dtype=torch.complex128, device=cuda)
    _, g128, _ = _loss_grad(c128, params, t)
    assert float(torch.linalg.vector_norm(g_p - g128)) <= 2e-5 * float(torch.linalg.vector_norm(g128))


def test_persistent_states_and_pingpong(cuda, persistent):
    gates, npar = qnn_gates(4, 2)
    params = torch.tensor(qnn_params(gates, npar, seed=5), device=cuda)
    circ = CompiledCircuit(4, 7, gates, npar, dtype=torch.complex64, device=cuda)
    all_states = circ.forward_states(params)
    final = circ.forward_states(params, store_all=False)
    assert torch.equal(all_states[circ.final_index()], final)
    assert circ.sweep_status() == (True, 0)
    # repeated sweeps on the same workspace keep working (barrier words reset)
    for _ in range(3):
        again = circ.forward_states(params, store_all=False)
        assert torch.equal(again, final)
    assert circ.sweep_status() == (True, 0)


def test_per_op_is_default(cuda, monkeypatch):
    monkeypatch.delenv("FOCK_GB300_SWEEP_MAX_BYTES", raising=False)
    gates, npar = qnn_gates(3, 1)
    circ = CompiledCircuit(3, 6, gates, npar, dtype=torch.complex64, device=cuda)
    assert circ.sweep_status() == (False, 0)


def test_persistent_graph_capture(cuda, persistent):
    from strawberryfields_gb300.autograd import GraphedGradient

    gates, npar = qnn_gates(3, 2)
    params = torch.tensor(qnn_params(gates, npar, seed=9), device=cuda)
    t = torch.as_tensor(target_state(3, 8, 3, 1), device=cuda).to(torch.complex64)
    circ = CompiledCircuit(3, 8, gates, npar, dtype=torch.complex64, device=cuda)

    def loss_fn(psi):
        s = torch.sum(t.conj() * psi)
        return 1 - (s.real ** 2 + s.imag ** 2)

    g = GraphedGradient(circ, loss_fn, params)
    loss, grad = g(params)
    _, g_eager, l_eager = _loss_grad(circ, params, t)
    assert abs(float(loss) - l_eager) < 1e-6
    assert float(torch.linalg.vector_norm(grad - g_eager)) <= 1e-6 * float(torch.linalg.vector_norm(g_eager))
    assert circ.sweep_status() == (True, 0)


def test_barrier_that_runs_out_sets_error_and_returns(cuda, persistent, monkeypatch):
    """A grid barrier with a spin limit too short for the other CTAs to arrive
    (FOCK_GB300_SWEEP_SPIN_LIMIT=0: one poll of the generation word) gives up:
    the kernel sets the error flag and returns, fock_plan_sweep_status reports
    it, and the device stays usable -- a plan with the default limit then runs
    the same sweep to the per-op result.  No trap and no unbounded wait: every
    CTA leaves at its next barrier."""
    gates, npar = qnn_gates(4, 2)
    params = torch.tensor(qnn_params(gates, npar, seed=6), device=cuda)
    monkeypatch.setenv("FOCK_GB300_SWEEP_SPIN_LIMIT", "0")
    short = CompiledCircuit(4, 8, gates, npar, dtype=torch.complex64, device=cuda)
    short.forward_states(params, store_all=False)
    pers, err = short.sweep_status()
    assert pers and err == 1
    monkeypatch.delenv("FOCK_GB300_SWEEP_SPIN_LIMIT")
    good = CompiledCircuit(4, 8, gates, npar, dtype=torch.complex64, device=cuda)
    psi = good.forward_states(params, store_all=False)
    pers, err = good.sweep_status()
    assert pers and err == 0
    monkeypatch.setenv("FOCK_GB300_SWEEP_MAX_BYTES", "0")
    ref = CompiledCircuit(4, 8, gates, npar, dtype=torch.complex64, device=cuda)
    assert torch.equal(psi, ref.forward_states(params, store_all=False))
