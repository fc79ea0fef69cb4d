"""A reference ``sf.Program`` with free parameters, compiled to the GB300
adjoint path (strawberryfields_gb300/program.py), against the hand-written
gate list of the same circuit and the oracle.

The program is the CV-QNN of the reference's training example
(examples/quantum_neural_network.py: ``interferometer`` :14-50, ``layer``
:55-85, free parameters from ``prog.params``), laid out so its gate order and
argument order equal ``qnn.qnn_gates``: then both compile to the same plan and
their gradients agree bit for bit.
"""
import numpy as np
import pytest

from oracle import fock_oracle as fo

pytestmark = pytest.mark.gpu


def _sf():
    pytest.importorskip("sympy")
    pytest.importorskip("networkx")
    from oracle import sfref

    try:
        return sfref.import_strawberryfields()
    except ImportError:
        pytest.skip("reference sources not available")


def qnn_program(sf, N, layers):
    """CV-QNN program: per layer a rectangular beamsplitter mesh on adjacent
    pairs with rotations on the first N-1 modes, squeezers, a second mesh,
    then displacement and Kerr on every mode; every argument a free
    parameter named p<k> in gate order."""
    from strawberryfields import ops

    prog = sf.Program(N)
    k = [0]

    def par(n):
        names = [f"p{k[0] + i}" for i in range(n)]
        k[0] += n
        return prog.params(*names)

    def mesh(q):
        for a in range(N):
            for j in range(N - 1):
                if (a + j) % 2 != 1:
                    theta, phi = par(2)
                    ops.BSgate(theta, phi) | (q[j], q[j + 1])
        for i in range(max(1, N - 1)):
            ops.Rgate(par(1)) | q[i]

    with prog.context as q:
        for _ in range(layers):
            mesh(q)
            for i in range(N):
                r, phi = par(2)
                ops.Sgate(r, phi) | q[i]
            mesh(q)
            for i in range(N):
                r, phi = par(2)
                ops.Dgate(r, phi) | q[i]
                ops.Kgate(par(1)) | q[i]
    return prog


@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
def test_program_gradients_equal_gate_list_and_oracle(cuda, dtype):
    import torch
    from strawberryfields_gb300 import CompiledCircuit
    from strawberryfields_gb300.program import ProgramCircuit
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params, target_state

    sf = _sf()
    N, D, layers = 3, 7, 2
    prog = qnn_program(sf, N, layers)
    tdt = torch.complex64 if dtype == "complex64" else torch.complex128
    pc = ProgramCircuit(prog, D, dtype=tdt)
    gates, npar = qnn_gates(N, layers)
    assert pc.program.gates == [tuple(g) for g in gates]
    params = qnn_params(gates, npar, seed=3)
    t = torch.as_tensor(target_state(N, D, 3, seed=4), device="cuda").to(tdt)

    def loss_of(psi):
        s = torch.sum(t.conj() * psi)
        return 1 - (s.real ** 2 + s.imag ** 2)

    # the reference's training call style: a mapping name -> value
    x = torch.tensor(params, device="cuda", requires_grad=True)
    mapping = {n: x[i] for i, n in enumerate(pc.free_params)}
    psi_prog = pc(mapping)
    loss_of(psi_prog).backward()
    g_prog = x.grad.clone()

    circ = CompiledCircuit(N, D, gates, npar, dtype=tdt)
    p = torch.tensor(params, device="cuda", requires_grad=True)
    psi = circ(p)
    loss_of(psi).backward()
    assert torch.equal(psi_prog, psi)
    assert torch.equal(g_prog, p.grad)

    ref = fo.run_gates(gates, params, N, D)[-1]
    tref = target_state(N, D, 3, seed=4)
    s = np.vdot(tref, ref)
    g_ref = fo.adjoint_grads(gates, params, N, D, -2 * s * tref)
    tol = 1e-10 if dtype == "complex128" else 1e-5
    assert np.linalg.norm(g_prog.cpu().numpy() - g_ref) <= tol * np.linalg.norm(g_ref)


def test_program_expressions_dagger_loss_and_batch(cuda):
    """Expressions of free parameters, a daggered gate, a loss channel (mixed
    state) and a batch of parameter sets, against the oracle's density-matrix
    runner and central differences of it."""
    import torch
    from strawberryfields import ops
    from strawberryfields_gb300.program import ProgramCircuit

    sf = _sf()
    N, D = 2, 6
    prog = sf.Program(N)
    with prog.context as q:
        ops.Coherent(0.3, 0.2) | q[1]
        a, b, T = prog.params("a", "b", "T")
        ops.Sgate(a, 0.4).H | q[0]
        ops.BSgate(2 * a, sf.math.sin(b)) | (q[0], q[1])
        ops.LossChannel(T) | q[1]
        ops.Dgate(b, -a) | q[0]
        ops.Rgate(0.0) | q[1]  # skipped, as the reference skips it
    B = 3
    pc = ProgramCircuit(prog, D, dtype=torch.complex128, batch_size=B)
    assert not pc.pure
    vals = np.array([[0.2, 0.5, 0.9], [0.1, 0.3, 0.8], [0.25, 0.7, 0.95]])
    x = torch.tensor(vals, device="cuda", requires_grad=True)
    rho = pc(x)
    n_vec = torch.arange(D, device="cuda", dtype=torch.float64)
    # loss: mean photon number of mode 0, summed over the batch
    diag0 = torch.diagonal(torch.diagonal(rho, dim1=3, dim2=4), dim1=1, dim2=2)  # [B, D(mode1), D(mode0)]
    loss = torch.sum(diag0.real.sum(dim=1) * n_vec)
    loss.backward()

    def oracle_rho(v):
        a, b, T = v
        gates = [(4, 0, -1, 0), (5, 0, 1, 2), (9, 1, -1, 4), (3, 0, -1, 5)]
        par = [-a, 0.4, 2 * a, np.sin(b), T, b, -a]
        psi = np.zeros((D, D), dtype=np.complex128)
        psi[0, :] = fo.coherent_state(0.3, 0.2, D)  # mode 0 in vacuum, mode 1 coherent
        return fo.run_gates_mixed(gates, par, N, D, rho=fo.mix(psi, N))

    def oracle_loss(v):
        return float(np.real(np.einsum("nnkk->n", oracle_rho(v))) @ np.arange(D))

    for bi in range(B):
        got = rho[bi].detach().cpu().numpy()
        assert np.abs(got - oracle_rho(vals[bi])).max() < 1e-12
        h = 1e-6
        fd = []
        for j in range(3):
            e = np.zeros(3)
            e[j] = h
            fd.append((oracle_loss(vals[bi] + e) - oracle_loss(vals[bi] - e)) / (2 * h))
        assert np.abs(x.grad[bi].cpu().numpy() - np.array(fd)).max() < 1e-7
