"""Fused tile groups of the forward sweep (csrc/tile.cu, on with
FOCK_GB300_TILE_GROUPS=1): a complex64 pure-state plan whose ops are grouped on
three-mode tiles against the same plan without groups (the default) and
against the complex128 sweep -- forward states, gradients (the adjoint sweep
reads the states the grouped forward stored), batches, checkpointed sweeps and
the captured graph.  Bars: states 1e-5; gradients 1e-5 relative L2."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _grad(circ, p, t, state_in=None):
    import torch

    p = p.detach().clone().requires_grad_(True)
    psi = circ(p, state_in)
    dims = tuple(range(psi.dim() - t.dim(), psi.dim()))
    s = torch.sum(t.to(psi.dtype).conj() * psi, dim=dims)
    torch.sum(1 - (s.real ** 2 + s.imag ** 2)).backward()
    return psi.detach(), p.grad.detach()


def _pair(monkeypatch, N, D, gates, npar, **kw):
    import torch
    from strawberryfields_gb300 import CompiledCircuit

    monkeypatch.setenv("FOCK_GB300_TILE_GROUPS", "1")
    grouped = CompiledCircuit(N, D, gates, npar, dtype=torch.complex64, **kw)
    monkeypatch.delenv("FOCK_GB300_TILE_GROUPS")
    plain = CompiledCircuit(N, D, gates, npar, dtype=torch.complex64, **kw)
    c128 = CompiledCircuit(N, D, gates, npar, dtype=torch.complex128, **kw)
    return grouped, plain, c128


def _n_groups(circ):
    import ctypes

    from strawberryfields_gb300 import _lib as L

    gs = set()
    for k in range(circ.n_ops):
        g = ctypes.c_int()
        L.check(L.load().fock_plan_op_group(circ._plan, k, ctypes.byref(g), None, None))
        if g.value >= 0:
            gs.add(g.value)
    return len(gs)


@pytest.mark.parametrize("N,D,layers,batch", [(6, 12, 2, 1), (7, 6, 2, 1), (6, 8, 2, 4), (5, 12, 1, 16),
                                              (6, 14, 1, 1), (5, 16, 1, 4)])
def test_grouped_matches_plain_and_fp64(cuda, monkeypatch, N, D, layers, batch):
    import torch
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params, target_state

    gates, npar = qnn_gates(N, layers)
    grouped, plain, c128 = _pair(monkeypatch, N, D, gates, npar, batch=batch)
    assert _n_groups(grouped) > 0 and _n_groups(plain) == 0
    if batch > 1:
        p = torch.stack([torch.tensor(qnn_params(gates, npar, seed=10 + i), device=cuda) for i in range(batch)])
    else:
        p = torch.tensor(qnn_params(gates, npar, seed=10), device=cuda)
    t = torch.as_tensor(target_state(N, D, 4, seed=3), device=cuda)
    psi_g, g_g = _grad(grouped, p, t)
    psi_p, g_p = _grad(plain, p, t)
    psi_d, g_d = _grad(c128, p, t)
    assert float(torch.max(torch.abs(psi_g - psi_p))) < 1e-5
    assert float(torch.max(torch.abs(psi_g.to(torch.complex128) - psi_d))) < 1e-5
    for a, b in ((g_g, g_p), (g_g, g_d.to(g_g.dtype))):
        assert float(torch.linalg.vector_norm(a - b)) <= 1e-5 * float(torch.linalg.vector_norm(b))
    # every op's stored output: the grouped forward writes what the per-op sweep writes
    sg = grouped.forward_states(p)
    # the groups reorder commuting ops, so compare the final states and the
    # checkpointed and ping-pong sweeps' final states
    assert float(torch.max(torch.abs(sg[grouped.final_index()] - psi_p))) < 1e-5
    fin0 = grouped.forward_states(p, store_all=False)
    assert float(torch.max(torch.abs(fin0 - psi_p))) < 1e-5


@pytest.fixture
def groups_on(monkeypatch):
    monkeypatch.setenv("FOCK_GB300_TILE_GROUPS", "1")


def test_grouped_checkpointed_and_recomputed(cuda, groups_on):
    """Checkpointed sweep (the grouped forward stores every k-th state; the
    adjoint recomputes segments with per-op launches) and a bounded
    recomputation pool."""
    import torch
    from strawberryfields_gb300 import CompiledCircuit
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params, target_state

    N, D = 6, 12
    gates, npar = qnn_gates(N, 2)
    p = torch.tensor(qnn_params(gates, npar, seed=21), device=cuda)
    t = torch.as_tensor(target_state(N, D, 4, seed=5), device=cuda)
    ref = CompiledCircuit(N, D, gates, npar, dtype=torch.complex64)
    assert _n_groups(ref) > 0
    _, g_ref = _grad(ref, p, t)
    for k, slots in ((7, None), (13, 3)):
        c = CompiledCircuit(N, D, gates, npar, dtype=torch.complex64, checkpoint=k, recompute_slots=slots)
        _, g = _grad(c, p, t)
        assert float(torch.linalg.vector_norm(g - g_ref)) <= 1e-5 * float(torch.linalg.vector_norm(g_ref))


def test_grouped_state_in_gradient_and_graph(cuda, monkeypatch):
    """dL/dstate_in of a grouped plan, and the whole step captured as one CUDA
    graph replaying the grouped launches."""
    import torch
    from strawberryfields_gb300.autograd import GraphedGradient
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params, target_state

    N, D = 6, 12
    gates, npar = qnn_gates(N, 1)
    grouped, plain, _ = _pair(monkeypatch, N, D, gates, npar)
    rng = np.random.default_rng(4)
    x = rng.normal(size=(D,) * N) + 1j * rng.normal(size=(D,) * N)
    x = torch.as_tensor(x / np.linalg.norm(x), device=cuda).to(torch.complex64)
    p = torch.tensor(qnn_params(gates, npar, seed=2), device=cuda)
    t = torch.as_tensor(target_state(N, D, 4, seed=6), device=cuda)
    grads_in = []
    for circ in (grouped, plain):
        xi = x.clone().requires_grad_(True)
        pp = p.clone().requires_grad_(True)
        psi = circ(pp, xi)
        s = torch.sum(t.to(psi.dtype).conj() * psi)
        (1 - (s.real ** 2 + s.imag ** 2)).backward()
        grads_in.append(xi.grad.detach())
    assert float(torch.linalg.vector_norm(grads_in[0] - grads_in[1])) <= 1e-5 * float(
        torch.linalg.vector_norm(grads_in[1]))

    def loss_fn(psi):
        s = torch.sum(t.to(psi.dtype).conj() * psi)
        return 1 - (s.real ** 2 + s.imag ** 2)

    gg = GraphedGradient(grouped, loss_fn, p)
    _, g_graph = gg(p)
    _, g_eager = _grad(grouped, p, t)
    assert torch.equal(g_graph, g_eager)
