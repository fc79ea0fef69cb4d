"""GPU compiled circuits (fused forward sweep) and adjoint gradients (rows
A1-A3) against the oracle's tape adjoint, itself pinned to central finite
differences in tests/test_oracle.py.

Bars: complex128 state max abs error <= 1e-12 and gradient relative L2 error
<= 1e-10; complex64 state <= 1e-5 and gradient relative L2 error <= 1e-5.
"""
import numpy as np
import pytest

from oracle import fock_oracle as fo

pytestmark = pytest.mark.gpu

# (kind, mode1, mode2, pidx) gate lists exercising every fusion rule
MIXED_LIST = [
    (1, 0, -1, 0),   # R before anything on mode 0 -> pre term of the BS
    (2, 2, -1, 1),   # K on mode 2 -> pre term of the S2 (slot b)
    (5, 0, 1, 2),
    (4, 1, -1, 4),
    (8, 0, 2, 6),    # cross-Kerr, flushed as its own op before S on 2
    (4, 2, -1, 7),
    (3, 0, -1, 9),
    (2, 0, -1, 11),  # K after D on mode 0 -> post term (last op on mode 0 later? no: BS below)
    (6, 2, 1, 12),   # S2 with swapped mode order
    (7, 0, 2, 14),   # MZ on a non-adjacent pair
    (8, 1, 2, 16),   # cross-Kerr fused into the next gate on the same pair
    (5, 1, 2, 17),
    (1, 1, -1, 19),  # trailing R on mode 1 -> post term of the last op on 1
    (2, 2, -1, 20),
]
MIXED_NPARAMS = 21


def _loss_grad(psi, t):
    s = np.vdot(t, psi)
    return 1 - abs(s) ** 2, -2 * s * t


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_fused_list_forward_and_gradient(cuda, dtype):
    import torch
    from strawberryfields_gb300 import CompiledCircuit

    N, D = 3, 6
    rng = np.random.default_rng(7)
    params = rng.uniform(0.05, 0.6, MIXED_NPARAMS)
    tdt = torch.complex128 if dtype == "complex128" else torch.complex64
    circ = CompiledCircuit(N, D, MIXED_LIST, MIXED_NPARAMS, dtype=tdt)
    assert circ.n_ops < len(MIXED_LIST)
    p = torch.tensor(params, device="cuda", requires_grad=True)
    psi = circ(p)
    ref_states = fo.run_gates(MIXED_LIST, params, N, D)
    tol = 1e-12 if dtype == "complex128" else 1e-5
    assert np.abs(psi.detach().to(torch.complex128).cpu().numpy() - ref_states[-1]).max() < tol
    t = rng.normal(size=(D,) * N) + 1j * rng.normal(size=(D,) * N)
    t /= np.linalg.norm(t)
    tt = torch.as_tensor(t, device="cuda").to(tdt)
    loss = 1 - torch.abs(torch.sum(tt.conj() * psi)) ** 2
    loss.backward()
    _, g_final = _loss_grad(ref_states[-1], t)
    ref = fo.adjoint_grads(MIXED_LIST, params, N, D, g_final)
    got = p.grad.cpu().numpy()
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel < (1e-10 if dtype == "complex128" else 1e-5), rel


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_qnn_forward_and_gradient(cuda, dtype):
    import torch
    from strawberryfields_gb300 import CompiledCircuit
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params, target_state

    N, D, layers = 4, 7, 2
    gates, npar = qnn_gates(N, layers)
    params = qnn_params(gates, npar, seed=3)
    tdt = torch.complex128 if dtype == "complex128" else torch.complex64
    circ = CompiledCircuit(N, D, gates, npar, dtype=tdt)
    # diagonal gates are fused away: one op per non-diagonal gate
    nd = sum(1 for g in gates if g[0] not in (1, 2, 8))
    assert circ.n_ops == nd
    p = torch.tensor(params, device="cuda", requires_grad=True)
    psi = circ(p)
    ref_states = fo.run_gates(gates, params, N, D)
    tol = 1e-12 if dtype == "complex128" else 1e-5
    assert np.abs(psi.detach().to(torch.complex128).cpu().numpy() - ref_states[-1]).max() < tol
    t = target_state(N, D, 4, seed=5)
    tt = torch.as_tensor(t, device="cuda").to(tdt)
    loss = 1 - torch.abs(torch.sum(tt.conj() * psi)) ** 2
    loss.backward()
    ref = fo.adjoint_grads(gates, params, N, D, _loss_grad(ref_states[-1], t)[1])
    got = p.grad.cpu().numpy()
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel < (1e-10 if dtype == "complex128" else 1e-5), rel


def test_gradient_vs_central_differences_of_gpu_forward(cuda):
    """The adjoint matches central differences of the GPU forward itself."""
    import torch
    from strawberryfields_gb300 import CompiledCircuit
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params, target_state

    N, D = 3, 6
    gates, npar = qnn_gates(N, 1)
    params = qnn_params(gates, npar, seed=11)
    circ = CompiledCircuit(N, D, gates, npar, dtype=torch.complex128)
    t = torch.as_tensor(target_state(N, D, 3, seed=2), device="cuda")

    def loss(pv):
        psi = circ.forward_states(torch.tensor(pv, device="cuda"), store_all=False)
        return float((1 - torch.abs(torch.sum(t.conj() * psi)) ** 2).item())

    p = torch.tensor(params, device="cuda", requires_grad=True)
    psi = circ(p)
    (1 - torch.abs(torch.sum(t.conj() * psi)) ** 2).backward()
    h = 1e-6
    fd = np.array([(loss(params + h * e) - loss(params - h * e)) / (2 * h) for e in np.eye(npar)])
    assert np.abs(p.grad.cpu().numpy() - fd).max() < 1e-8


def test_known_gradients_beamsplitter_on_11(cuda):
    """Closed forms of the reference's TF gradient tests
    (tests/integration/test_tf_integration.py: BS on |1,1>):
    dP11/dtheta = -4 sin(2 theta) cos(2 theta), dP02/dtheta = sin(4 theta)."""
    import torch
    from strawberryfields_gb300 import CompiledCircuit

    D = 4
    theta = 0.37
    circ = CompiledCircuit(2, D, [(5, 0, 1, 0)], 2, dtype=torch.complex128)
    psi0 = torch.zeros((D, D), dtype=torch.complex128, device="cuda")
    psi0[1, 1] = 1.0
    for idx, ref in [((1, 1), -4 * np.sin(2 * theta) * np.cos(2 * theta)), ((0, 2), np.sin(4 * theta))]:
        p = torch.tensor([theta, 0.0], device="cuda", dtype=torch.float64, requires_grad=True)
        psi = circ(p, state_in=psi0)
        prob = torch.abs(psi[idx]) ** 2
        prob.backward()
        assert abs(p.grad[0].item() - ref) < 1e-12


def test_known_gradient_two_mode_squeeze_vacuum(cuda):
    """dP00/dr = -2 tanh(r) / cosh(r)^2 for S2(r)|00> (test_tf_integration.py)."""
    import torch
    from strawberryfields_gb300 import CompiledCircuit

    r = 0.21
    circ = CompiledCircuit(2, 6, [(6, 0, 1, 0)], 2, dtype=torch.complex128)
    p = torch.tensor([r, 0.3], device="cuda", dtype=torch.float64, requires_grad=True)
    psi = circ(p)
    (torch.abs(psi[0, 0]) ** 2).backward()
    assert abs(p.grad[0].item() + 2 * np.tanh(r) / np.cosh(r) ** 2) < 1e-12


def test_known_gradient_displacement_mean_photon(cuda):
    """d<n>/dr = 2 r for a coherent state (high cutoff), d/dphi = 0."""
    import torch
    from strawberryfields_gb300 import CompiledCircuit

    D, r = 20, 0.4
    circ = CompiledCircuit(1, D, [(3, 0, -1, 0)], 2, dtype=torch.complex128)
    p = torch.tensor([r, 0.8], device="cuda", dtype=torch.float64, requires_grad=True)
    psi = circ(p)
    n = torch.arange(D, device="cuda", dtype=torch.float64)
    (torch.sum(n * torch.abs(psi) ** 2)).backward()
    assert abs(p.grad[0].item() - 2 * r) < 1e-9
    assert abs(p.grad[1].item()) < 1e-12


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_batched_circuits_match_individual_runs(cuda, dtype):
    """B circuits of one structure with their own parameters (TF batch axis)."""
    import torch
    from strawberryfields_gb300 import CompiledCircuit
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params, target_state

    N, D, B = 3, 6, 5
    gates, npar = qnn_gates(N, 2)
    P = np.stack([qnn_params(gates, npar, seed=20 + b) for b in range(B)])
    tdt = torch.complex128 if dtype == "complex128" else torch.complex64
    circ = CompiledCircuit(N, D, gates, npar, dtype=tdt, batch=B)
    p = torch.tensor(P, device="cuda", requires_grad=True)
    psi = circ(p)
    assert tuple(psi.shape) == (B,) + (D,) * N
    t = target_state(N, D, 3, seed=4)
    tt = torch.as_tensor(t, device="cuda").to(tdt)
    s = torch.sum(tt.conj() * psi, dim=tuple(range(1, N + 1)))
    (1 - torch.abs(s) ** 2).sum().backward()
    tol = 1e-12 if dtype == "complex128" else 1e-5
    for b in range(B):
        ref_states = fo.run_gates(gates, P[b], N, D)
        assert np.abs(psi[b].detach().to(torch.complex128).cpu().numpy() - ref_states[-1]).max() < tol
        ref = fo.adjoint_grads(gates, P[b], N, D, _loss_grad(ref_states[-1], t)[1])
        rel = np.linalg.norm(p.grad[b].cpu().numpy() - ref) / np.linalg.norm(ref)
        assert rel < (1e-10 if dtype == "complex128" else 1e-5), (b, rel)


@pytest.mark.parametrize("k", [2, 3, 7])
def test_checkpointed_adjoint_matches_stored(cuda, k):
    """Keeping every k-th state and recomputing segments gives the same gradient."""
    import torch
    from strawberryfields_gb300 import CompiledCircuit
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params, target_state

    N, D = 3, 6
    gates, npar = qnn_gates(N, 2)
    params = qnn_params(gates, npar, seed=8)
    t = torch.as_tensor(target_state(N, D, 3, seed=9), device="cuda")
    out = []
    for kk in (1, k):
        circ = CompiledCircuit(N, D, gates, npar, dtype=torch.complex128, checkpoint=kk)
        p = torch.tensor(params, device="cuda", requires_grad=True)
        psi = circ(p)
        (1 - torch.abs(torch.sum(t.conj() * psi)) ** 2).backward()
        out.append((psi.detach().cpu().numpy(), p.grad.cpu().numpy()))
    assert np.abs(out[0][0] - out[1][0]).max() < 1e-13
    assert np.abs(out[0][1] - out[1][1]).max() < 1e-12


@pytest.mark.parametrize("D", [3, 7, 11, 14, 19, 23, 26])
def test_gradient_every_cutoff_bucket(cuda, D):
    """Forward and adjoint parity in every compiled cutoff bucket (4, 8, 12,
    16, 20, 24) and on the generic path beyond 24, complex128 and complex64:
    dense single-mode ops, beamsplitters on an inner pair and on the last
    pair (plane kernels up to cutoff 16), a swapped two-mode squeezer."""
    import torch
    from strawberryfields_gb300 import CompiledCircuit

    N = 3
    gates = [(4, 0, -1, 0), (3, 2, -1, 2), (5, 0, 1, 4), (5, 1, 2, 6), (6, 2, 0, 8), (1, 1, -1, 10),
             (3, 1, -1, 11), (5, 2, 1, 13)]
    npar = 15
    rng = np.random.default_rng(D)
    params = rng.uniform(0.05, 0.35, npar)
    t = rng.normal(size=(D,) * N) + 1j * rng.normal(size=(D,) * N)
    t /= np.linalg.norm(t)
    ref_states = fo.run_gates(gates, params, N, D)
    _, g_final = _loss_grad(ref_states[-1], t)
    ref = fo.adjoint_grads(gates, params, N, D, g_final)
    for tdt, tol_s, tol_g in ((torch.complex128, 1e-11, 1e-9), (torch.complex64, 1e-5, 1e-4)):
        circ = CompiledCircuit(N, D, gates, npar, dtype=tdt)
        p = torch.tensor(params, device="cuda", requires_grad=True)
        psi = circ(p)
        assert np.abs(psi.detach().to(torch.complex128).cpu().numpy() - ref_states[-1]).max() < tol_s
        tt = torch.as_tensor(t, device="cuda").to(tdt)
        loss = 1 - torch.abs(torch.sum(tt.conj() * psi)) ** 2
        loss.backward()
        got = p.grad.cpu().numpy()
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < tol_g, (D, tdt)


def test_backward_reuses_or_rebuilds_matrices(cuda):
    """The adjoint sweep reuses the forward sweep's matrices only when the
    workspace still holds them for the same, unmodified parameters."""
    import torch
    from strawberryfields_gb300 import CompiledCircuit
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params

    gates, npar = qnn_gates(3, 2)
    p1 = torch.tensor(qnn_params(gates, npar, seed=1), device="cuda")
    p2 = torch.tensor(qnn_params(gates, npar, seed=2), device="cuda")
    g_state = torch.randn(6, 6, 6, dtype=torch.complex128, device="cuda")

    def fresh(p):
        c = CompiledCircuit(3, 6, gates, npar, dtype=torch.complex128)
        s = c.forward_states(p)
        return c.backward(p, s, g_state)[0]

    ref1, ref2 = fresh(p1), fresh(p2)
    c = CompiledCircuit(3, 6, gates, npar, dtype=torch.complex128)
    s1 = c.forward_states(p1)
    s2 = c.forward_states(p2)  # the workspace now holds p2's matrices
    assert torch.allclose(c.backward(p1, s1, g_state)[0], ref1, rtol=1e-12, atol=1e-14)
    s2 = c.forward_states(p2)
    assert torch.allclose(c.backward(p2, s2, g_state)[0], ref2, rtol=1e-12, atol=1e-14)  # reused
    s1 = c.forward_states(p1)
    p1.mul_(1.0)  # in-place update: version changes, matrices rebuilt
    assert torch.allclose(c.backward(p1, s1, g_state)[0], ref1, rtol=1e-12, atol=1e-14)


def test_tuned_kernels_give_the_same_gradient(cuda):
    """Every kernel family and adjoint CTA density of fock_plan_tune, and the
    autotuner's pick, give the untuned gradient (complex128: only the order
    of the partial sums changes)."""
    import torch
    from strawberryfields_gb300 import CompiledCircuit
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params

    N, D = 4, 9
    gates, npar = qnn_gates(N, 2)
    p = torch.tensor(qnn_params(gates, npar, seed=3), device="cuda")
    g_state = torch.randn([D] * N, dtype=torch.complex128, device="cuda")
    c = CompiledCircuit(N, D, gates, npar, dtype=torch.complex128)
    ref_s = c.forward_states(p)
    ref_g = c.backward(p, ref_s, g_state)[0]
    start = [c.op_config(k) for k in range(c.n_ops)]
    assert any(ok for _, _, ok, _ in start)
    for fam, ctas, tc in [(0, 1, 0), (0, 3, 0), (0, 16, 0), (1, 0, 0), (1, 0, 24), (1, 0, 8)]:
        for k in range(c.n_ops):
            two = start[k][2] and start[k][3] <= 32
            c.tune_op(k, fam if (fam == 0 or start[k][2]) else 0, ctas, tc if two else 0)
        s = c.forward_states(p)
        assert torch.allclose(s, ref_s, rtol=0, atol=1e-13), (fam, ctas, tc)
        g = c.backward(p, s, g_state)[0]
        assert torch.allclose(g, ref_g, rtol=1e-11, atol=1e-13), (fam, ctas, tc)
    configs, before, after = c.autotune(p, ctas=(2, 8), tiles=(32, 16), repeats=1)
    assert len(configs) == c.n_ops and after <= before
    s = c.forward_states(p)
    g = c.backward(p, s, g_state)[0]
    assert torch.allclose(s, ref_s, rtol=0, atol=1e-13)
    assert torch.allclose(g, ref_g, rtol=1e-11, atol=1e-13)


@pytest.mark.parametrize("D", [3, 4, 7, 12, 16, 20])
@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_plane_kernels_on_every_op_match_oracle(cuda, D, dtype):
    """Every op that has a plane-tile kernel switched to it (inner and last
    axes, one- and two-mode, cutoffs up to the plane limits 16 / 24; small
    cutoffs exercise the column-group split of the adjoint's C pass) against
    the oracle's tape adjoint."""
    import torch
    from strawberryfields_gb300 import CompiledCircuit
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params

    N = 3
    gates, npar = qnn_gates(N, 1)
    params = qnn_params(gates, npar, seed=D)
    tdt = getattr(torch, dtype)
    circ = CompiledCircuit(N, D, gates, npar, dtype=tdt)
    n_plane = 0
    for k in range(circ.n_ops):
        if circ.op_config(k)[2]:
            circ.tune_op(k, 1, 0)
            n_plane += 1
    assert n_plane > 0
    rng = np.random.default_rng(D)
    t = rng.normal(size=(D,) * N) + 1j * rng.normal(size=(D,) * N)
    t /= np.linalg.norm(t)
    p = torch.tensor(params, device="cuda", dtype=torch.float64, requires_grad=True)
    psi = circ(p)
    tt = torch.as_tensor(t, device="cuda").to(tdt)
    (1 - torch.abs(torch.sum(tt.conj() * psi)) ** 2).backward()
    ref_states = fo.run_gates(gates, params, N, D)
    s = np.vdot(t, ref_states[-1])
    ref = fo.adjoint_grads(gates, params, N, D, -2 * s * t)
    tol_s, tol_g = (1e-12, 1e-10) if dtype == "complex128" else (1e-5, 1e-5)
    assert np.abs(psi.detach().to(torch.complex128).cpu().numpy() - ref_states[-1]).max() < tol_s
    got = p.grad.cpu().numpy()
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < tol_g


def test_state_at_an_8_byte_offset(cuda):
    """A complex64 input state that starts 8 bytes past a 16-byte boundary
    (a slice of a larger buffer): the one-mode op on the innermost axis
    takes its 8-byte path there and gives the oracle's result."""
    import torch
    from strawberryfields_gb300 import CompiledCircuit

    N, D = 3, 6
    gates = [(4, 2, -1, 0), (5, 1, 2, 2)]  # squeezer on the last mode, then a beamsplitter
    params = np.array([0.3, 0.7, 0.5, 0.2])
    rng = np.random.default_rng(4)
    psi = rng.normal(size=(D,) * N) + 1j * rng.normal(size=(D,) * N)
    psi /= np.linalg.norm(psi)
    big = torch.zeros(D ** N + 1, dtype=torch.complex64, device="cuda")
    big[1:] = torch.as_tensor(psi.reshape(-1), device="cuda").to(torch.complex64)
    x = big[1:].reshape([D] * N)
    assert x.data_ptr() % 16 == 8
    circ = CompiledCircuit(N, D, gates, 4, dtype=torch.complex64)
    p = torch.tensor(params, device="cuda", dtype=torch.float64)
    out = circ.forward_states(p, state_in=x, store_all=False)
    ref = fo.run_gates(gates, params, N, D, psi)[-1]
    assert np.abs(out.to(torch.complex128).cpu().numpy() - ref).max() < 1e-5
