"""The workload configurations at their full sizes against the oracle:

* 6-mode cutoff-12 CV-QNN forward (4 layers, 12^6 = 3.0M amplitudes), complex128
  and complex64, with the fock_prob and mean_photon readouts;
* 4-mode cutoff-15 CV-QNN adjoint gradient (8 layers, 400 parameters,
  loss 1 - |<psi_t|psi>|^2 with a target of total photon number <= 6),
  complex64 and complex128, against the oracle's tape adjoint (itself pinned
  to central differences in tests/test_oracle.py).

Bars: states 1e-12 (complex128) / 1e-5 (complex64) max abs; gradients 1e-10 /
1e-5 relative L2.
"""
import numpy as np
import pytest

from oracle import fock_oracle as fo

pytestmark = pytest.mark.gpu


def _oracle_final(gates, params, N, D):
    """Final pure state of a gate list, keeping one state at a time."""
    psi = fo.vacuum(N, D)
    for kind, m1, m2, pi in gates:
        p = [params[pi + k] for k in range(fo.NPARAMS[kind])]
        U, _ = fo.gate_matrix(kind, p, D)
        psi = fo.apply_gate1(psi, U, m1) if U.ndim == 2 else fo.apply_gate2(psi, U, m1, m2)
    return psi


@pytest.fixture(scope="module")
def qnn6x12():
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params

    gates, npar = qnn_gates(6, 4)
    params = qnn_params(gates, npar, seed=0)
    return gates, npar, params, _oracle_final(gates, params, 6, 12)


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_qnn6x12_forward_and_readouts(cuda, qnn6x12, dtype):
    import torch
    from strawberryfields_gb300 import CompiledCircuit
    from strawberryfields_gb300.states import FockStateGB300

    gates, npar, params, ref = qnn6x12
    tdt = getattr(torch, dtype)
    circ = CompiledCircuit(6, 12, gates, npar, dtype=tdt)
    psi = circ(torch.tensor(params, device="cuda", dtype=torch.float64))
    tol = 1e-12 if dtype == "complex128" else 1e-5
    got = psi.detach().to(torch.complex128).cpu().numpy()
    assert np.abs(got - ref).max() < tol
    st = FockStateGB300(psi.detach(), 6, True, 12)
    n = [1, 0, 2, 0, 0, 1]
    assert abs(st.fock_prob(n) - abs(ref[tuple(n)]) ** 2) < tol
    tol_m = 1e-10 if dtype == "complex128" else 1e-4
    for m in (0, 5):
        mean, var = st.mean_photon(m)
        rm, rv = fo.mean_photon(ref, 6, m)
        assert abs(mean - rm) < tol_m and abs(var - rv) < tol_m


@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
def test_qnn4x15_adjoint_gradient(cuda, dtype):
    import torch
    from strawberryfields_gb300 import CompiledCircuit
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params, target_state

    N, D = 4, 15
    gates, npar = qnn_gates(N, 8)
    assert npar == 400
    params = qnn_params(gates, npar, seed=1)
    t = target_state(N, D, 6, seed=2)
    tdt = getattr(torch, dtype)
    circ = CompiledCircuit(N, D, gates, npar, dtype=tdt)
    p = torch.tensor(params, device="cuda", dtype=torch.float64, requires_grad=True)
    psi = circ(p)
    tt = torch.as_tensor(t, device="cuda").to(tdt)
    (1 - torch.abs(torch.sum(tt.conj() * psi)) ** 2).backward()
    states = fo.run_gates(gates, params, N, D)
    s = np.vdot(t, states[-1])
    ref = fo.adjoint_grads(gates, params, N, D, -2 * s * t)
    tol_s, tol_g = (1e-12, 1e-10) if dtype == "complex128" else (1e-5, 1e-5)
    assert np.abs(psi.detach().to(torch.complex128).cpu().numpy() - states[-1]).max() < tol_s
    got = p.grad.cpu().numpy()
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < tol_g
