"""The ``fock_gb300`` backend through its ``BaseFock`` API, in the style of the
reference's backend tests (``tests/backend/*``: the backend class is driven
directly), with the reference's analytic known answers and oracle parity of
gate sequences (complex128: 1e-12; complex64: 1e-5).
"""
import math

import numpy as np
import pytest

from oracle import fock_oracle as fo

pytestmark = pytest.mark.gpu

ALPHA = 0.1
TOL = 1e-12


def make_backend(n, cutoff, pure=True, dtype="complex128"):
    from strawberryfields_gb300 import FockGB300Backend

    b = FockGB300Backend()
    b.begin_circuit(n, cutoff_dim=cutoff, pure=pure, dtype=dtype)
    return b


def coherent(alpha, D):
    k = np.arange(D)
    fac = np.array([math.factorial(int(i)) for i in k], dtype=float)
    return np.exp(-0.5 * abs(alpha) ** 2) * alpha ** k / np.sqrt(fac)


@pytest.mark.parametrize("pure", [True, False])
def test_displacement_column_is_coherent(cuda, pure):
    """test_displacement_operation.py:74-94: D(alpha)|0> = coherent amplitudes."""
    D = 8
    for r, phi in [(0.0, 0.0), (0.1, 0.3), (0.35, 2.2)]:
        b = make_backend(1, D, pure)
        b.displacement(r, phi, 0)
        ref = coherent(r * np.exp(1j * phi), D)
        st = b.state()
        if pure:
            assert np.abs(st.ket() - ref).max() < TOL
        else:
            assert np.abs(st.dm() - np.outer(ref, ref.conj())).max() < TOL


def test_squeezed_vacuum(cuda):
    """Loudon 5.5.6 (test_squeeze_operation.py:105-139)."""
    D = 10
    r, phi = 0.3, 0.7
    b = make_backend(1, D)
    b.squeeze(r, phi, 0)
    ref = np.zeros(D, dtype=complex)
    for n in range(0, D, 2):
        m = n // 2
        ref[n] = (math.sqrt(math.factorial(2 * m)) / (2 ** m * math.factorial(m))
                  * (-np.exp(1j * phi) * np.tanh(r)) ** m) / math.sqrt(math.cosh(r))
    assert np.abs(b.state().ket() - ref).max() < TOL


def test_two_mode_squeezed_vacuum(cuda):
    """TMSV amplitudes (e^{i phi} tanh r)^k / cosh r (test_twomode_squeezing_operation.py:32-47)."""
    D = 8
    r, phi = 0.2, 1.1
    for modes in [(0, 1), (1, 0)]:
        b = make_backend(2, D)
        b.two_mode_squeeze(r, phi, *modes)
        ket = b.state().ket()
        ref = np.zeros((D, D), dtype=complex)
        for k in range(D):
            ref[k, k] = (np.exp(1j * phi) * np.tanh(r)) ** k / np.cosh(r)
        assert np.abs(ket - ref).max() < TOL


def test_beamsplitter_coherent(cuda):
    """BS|alpha,0> = |t alpha, r alpha> (test_beamsplitter_operation.py:95-137),
    checked on the probabilities where truncation is negligible."""
    D = 14
    theta, phi = 0.6, 0.9
    a = 0.3
    b = make_backend(2, D)
    b.prepare_coherent_state(a, 0.0, 0)
    b.beamsplitter(theta, phi, 0, 1)
    st = b.state()
    t, rr = np.cos(theta), np.exp(1j * phi) * np.sin(theta)
    ref = np.outer(coherent(t * a, D), coherent(rr * a, D))
    # prepare_* on a multimode circuit mixes the state, as in the reference
    assert not st.is_pure
    probs = st.all_fock_probs()
    assert np.abs(probs - np.abs(ref) ** 2).max() < 1e-12


def test_loss_on_coherent(cuda):
    """Loss maps |alpha> to |sqrt(T) alpha> (test_loss_channel.py:175-207); T=0 gives vacuum."""
    D = 12
    a, T = 0.4 * np.exp(0.5j), 0.7
    b = make_backend(1, D)
    b.displacement(abs(a), np.angle(a), 0)
    b.loss(T, 0)
    ref = coherent(np.sqrt(T) * a, D)
    dm = b.state().dm()
    # analytic answer up to the truncation of the input state; oracle exactly
    assert np.abs(dm - np.outer(ref, ref.conj())).max() < 1e-9
    orc = fo.apply_loss(fo.apply_gate1(fo.vacuum(1, D), fo.displacement(abs(a), np.angle(a), D), 0), T, 0, 1, True)
    assert np.abs(dm - orc).max() < 1e-12
    b.loss(0.0, 0)
    dm = b.state().dm()
    assert abs(dm[0, 0] - 1) < 1e-12 and np.abs(dm).sum() - 1 < 1e-12


def test_diagonal_gates(cuda):
    """R = e^{i theta n}, K = e^{i kappa n^2}, CK = e^{i kappa n1 n2}
    (test_rotation_operation.py:57-80, test_nongaussian_gates.py:64-102)."""
    D = 6
    rng = np.random.default_rng(3)
    psi = rng.normal(size=(D, D)) + 1j * rng.normal(size=(D, D))
    psi /= np.linalg.norm(psi)
    b = make_backend(2, D)
    b.prepare_ket_state(psi, [0, 1])
    b.rotation(0.3, 0)
    b.kerr_interaction(0.07, 1)
    b.cross_kerr_interaction(0.11, 0, 1)
    n = np.arange(D)
    ref = psi * np.exp(1j * 0.3 * n)[:, None] * np.exp(1j * 0.07 * n ** 2)[None, :] * np.exp(1j * 0.11 * np.outer(n, n))
    assert np.abs(b.state().ket() - ref).max() < TOL


def _oracle_sequence(ops, N, D, pure):
    s = fo.vacuum(N, D, pure)
    for op in ops:
        name, args = op[0], op[1:]
        if name == "S":
            s = fo.apply_gate1(s, fo.squeezing(args[0], args[1], D), args[2], pure)
        elif name == "D":
            s = fo.apply_gate1(s, fo.displacement(args[0], args[1], D), args[2], pure)
        elif name == "R":
            s = fo.apply_gate1(s, fo.phase(args[0], D), args[1], pure)
        elif name == "K":
            s = fo.apply_gate1(s, fo.kerr(args[0], D), args[1], pure)
        elif name == "BS":
            s = fo.apply_gate2(s, fo.beamsplitter(args[0], args[1], D), args[2], args[3], pure)
        elif name == "S2":
            s = fo.apply_gate2(s, fo.two_mode_squeeze(args[0], args[1], D), args[2], args[3], pure)
        elif name == "MZ":
            s = fo.apply_gate2(s, fo.mzgate(args[0], args[1], D), args[2], args[3], pure)
        elif name == "CK":
            s = fo.apply_gate2(s, fo.cross_kerr(args[0], D), args[1], args[2], pure)
        elif name == "L":
            s = fo.apply_loss(s, args[0], args[1], N, pure)
            pure = False
    return s, pure


def _run_backend(b, ops):
    for op in ops:
        name, args = op[0], op[1:]
        {"S": b.squeeze, "D": b.displacement, "R": b.rotation, "K": b.kerr_interaction,
         "BS": b.beamsplitter, "S2": b.two_mode_squeeze, "MZ": b.mzgate, "CK": b.cross_kerr_interaction,
         "L": b.loss}[name](*args)


SEQ = [("S", 0.2, 0.4, 0), ("D", 0.3, 1.0, 1), ("R", 0.7, 0), ("BS", 0.5, 0.3, 0, 1), ("K", 0.05, 2),
       ("S2", 0.15, 0.2, 2, 1), ("CK", 0.09, 0, 2), ("MZ", 0.4, 1.3, 2, 0), ("D", 0.2, -0.5, 0),
       ("R", -0.3, 1), ("BS", 1.1, 2.0, 1, 2), ("K", 0.02, 0)]


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
@pytest.mark.parametrize("pure", [True, False])
def test_gate_sequence_matches_oracle(cuda, pure, dtype):
    N, D = 3, 6
    b = make_backend(N, D, pure, dtype)
    _run_backend(b, SEQ)
    ref, rpure = _oracle_sequence(SEQ, N, D, pure)
    st = b.state()
    tol = TOL if dtype == "complex128" else 1e-5
    got = st.ket() if pure else st.dm()
    assert np.abs(got.astype(np.complex128) - ref).max() < tol
    # readouts
    assert abs(st.trace() - (np.vdot(ref, ref).real if pure else fo.all_fock_probs(ref, N, False).sum())) < 100 * tol
    for m in range(N):
        mean, var = st.mean_photon(m)
        rm, rv = fo.mean_photon(ref, N, m, pure)
        assert abs(mean - rm) < tol * 10 and abs(var - rv) < tol * 100
        assert np.abs(st.reduced_dm(m) - fo.reduced_dm(ref, N, m, pure)).max() < tol
    assert abs(st.fock_prob([1, 0, 2]) - fo.all_fock_probs(ref, N, pure)[1, 0, 2]) < tol


def test_sequence_with_loss_goes_mixed(cuda):
    N, D = 2, 6
    seq = [("S", 0.3, 0.1, 0), ("BS", 0.7, 0.2, 0, 1), ("L", 0.8, 1), ("D", 0.2, 0.3, 0), ("K", 0.1, 1),
           ("BS", 0.3, 1.0, 1, 0), ("L", 0.9, 0)]
    b = make_backend(N, D, True)
    _run_backend(b, seq)
    ref, rpure = _oracle_sequence(seq, N, D, True)
    st = b.state()
    assert not st.is_pure and not rpure
    assert np.abs(st.dm() - ref).max() < TOL


def test_reduced_state_and_modes(cuda):
    N, D = 3, 5
    b = make_backend(N, D)
    _run_backend(b, SEQ[:6])
    ref, _ = _oracle_sequence(SEQ[:6], N, D, True)
    rho = fo.mix(ref, N)
    red = b.state(modes=[2, 0])
    # reference semantics: reduced dm of modes [2, 0] in that order (fockbackend/backend.py:209-264)
    r = np.trace(rho, axis1=2, axis2=3)  # trace mode 1 -> axes (k0, b0, k2, b2)
    r = np.transpose(r, (2, 3, 0, 1))
    assert np.abs(red.dm() - r).max() < TOL
    with pytest.raises(ValueError):
        b.state(modes=[0, 0])
    with pytest.raises(ValueError):
        b.displacement(0.1, 0.0, 7)


def test_prepare_and_measure_fock(cuda):
    N, D = 2, 5
    b = make_backend(N, D)
    b.prepare_fock_state(2, 0)
    b.prepare_fock_state(1, 1)
    probs = b.state().all_fock_probs()
    assert abs(probs[2, 1] - 1) < TOL
    res = b.measure_fock([0, 1])
    assert list(res[0]) == [2, 1]
    # after measurement the measured modes are reset to vacuum
    assert abs(b.state().all_fock_probs()[0, 0] - 1) < TOL


def test_coherent_fidelity_and_quadratures(cuda):
    D = 15
    a = 0.3 + 0.2j
    b = make_backend(1, D)
    b.displacement(abs(a), np.angle(a), 0)
    st = b.state()
    assert abs(st.fidelity_coherent([a]) - 1) < 1e-10
    mean, var = st.quad_expectation(0)
    assert abs(mean - 2 * a.real) < 1e-8 and abs(var - 1.0) < 1e-8  # hbar = 2
    assert abs(st.mean_photon(0)[0] - abs(a) ** 2) < 1e-10


def test_engine_integration(cuda):
    """An unchanged sf.Engine program on the backend (needs the reference's
    frontend dependencies networkx and sympy)."""
    pytest.importorskip("networkx")
    pytest.importorskip("sympy")
    from oracle import sfref

    try:
        sf = sfref.import_strawberryfields()
    except ImportError:
        pytest.skip("reference sources not available")
    from strawberryfields import ops as O
    from strawberryfields_gb300 import sf_backend

    prog = sf.Program(3)
    with prog.context as q:
        O.Sgate(0.2, 0.4) | q[0]
        O.Dgate(0.3, 1.0) | q[1]
        O.Rgate(0.7) | q[0]
        O.BSgate(0.5, 0.3) | (q[0], q[1])
        O.Kgate(0.05) | q[2]
        O.S2gate(0.15, 0.2) | (q[2], q[1])
    eng = sf.Engine(sf_backend(), backend_options={"cutoff_dim": 6})
    st = eng.run(prog).state
    ref, _ = _oracle_sequence(SEQ[:6], 3, 6, True)
    assert np.abs(st.ket() - ref).max() < TOL


@pytest.mark.parametrize("pure", [True, False])
@pytest.mark.parametrize("gamma", [-0.3, 0.1, 0.45])
def test_cubic_phase_matches_reference_known_answer(cuda, pure, gamma):
    """Cubic phase exp(i gamma x^3 / (3 hbar)) (reference fockbackend/ops.py:
    296-306, built at the cutoff, hbar = 2) on the uniform superposition, on a
    mode of a 2-mode state, against the known answer of the reference's
    tests/backend/test_nongaussian_gates.py:32-62 (x = a + a^dagger unscaled,
    exp(i gamma x^3 / 6)) at 1e-12."""
    from scipy.linalg import expm

    from strawberryfields_gb300 import FockGB300Backend

    D = 7
    b = FockGB300Backend()
    b.begin_circuit(2, cutoff_dim=D, pure=pure)
    ket = np.ones(D) / np.sqrt(D)
    b.prepare_ket_state(ket, 1)
    b.displacement(0.2, 0.4, 0)
    b.cubic_phase(gamma, 1)
    a = np.diag(np.sqrt(np.arange(1, D)), 1)
    x = a + a.T
    ref1 = expm(1j * gamma * (x @ x @ x) / 6) @ ket
    ref0 = fo.displacement(0.2, 0.4, D)[:, 0]
    st = b.state()
    got = st.dm() if not st.is_pure else np.multiply.outer(st.ket(), st.ket().conj()).transpose(0, 2, 1, 3)
    ref = np.multiply.outer(np.multiply.outer(ref0, ref0.conj()), np.multiply.outer(ref1, ref1.conj()))
    assert np.abs(got - ref).max() < TOL


@pytest.mark.parametrize("pure", [True, False])
def test_add_and_delete_modes_match_reference_backend(cuda, pure):
    """add_mode / del_mode / get_modes against the reference's own
    FockBackend (fockbackend/backend.py:130-139) on the same call sequence:
    modes appended in the vacuum, deleted modes traced out, labels of the
    remaining modes unchanged."""
    from oracle import sfref

    try:
        sfref.import_strawberryfields()
    except ImportError:
        pytest.skip("reference sources not available")
    from strawberryfields.backends.fockbackend import FockBackend
    from strawberryfields_gb300 import FockGB300Backend

    D = 5
    results = []
    for cls in (FockBackend, FockGB300Backend):
        b = cls()
        b.begin_circuit(2, cutoff_dim=D, pure=pure)
        b.squeeze(0.3, 0.2, 0)
        b.displacement(0.4, 1.1, 1)
        b.add_mode(2)
        b.beamsplitter(0.7, 0.3, 1, 3)
        b.two_mode_squeeze(0.2, 0.5, 0, 2)
        b.del_mode([1])
        b.kerr_interaction(0.1, 3)
        b.beamsplitter(0.4, 0.9, 0, 3)
        modes = b.get_modes()
        b.add_mode(1)
        b.displacement(0.2, 0.3, 4)
        b.del_mode(0)
        results.append((modes, b.get_modes(), b.state().dm(), b.state(modes=[2, 1]).dm()))
        with pytest.raises(ValueError):
            b.displacement(0.1, 0.0, 1)  # deleted label
        with pytest.raises(ValueError):
            b.del_mode([0])  # deleted already
    (m_ref, m2_ref, rho_ref, red_ref), (m_got, m2_got, rho_got, red_got) = results
    assert m_got == m_ref == [0, 2, 3]
    assert m2_got == m2_ref == [2, 3, 4]
    assert rho_got.shape == rho_ref.shape
    assert np.abs(rho_got - rho_ref).max() < TOL
    assert np.abs(red_got - red_ref).max() < TOL


@pytest.mark.parametrize("pure", [True, False])
@pytest.mark.parametrize("state,eps,D", [([0, 0], 0.2, 12), ([np.pi / 2, 0.4], 0.3, 20), ([1.1, 2.0], 0.25, 30)])
def test_gkp_matches_reference_backend(cuda, pure, state, eps, D):
    """prepare_gkp against the reference's FockBackend (fockbackend/backend.py:
    297-329, square lattice, real representation) on the second mode of a
    two-mode state, at 1e-8 (the device builds each tooth's displaced
    squeezed vacuum at cutoff 64, the reference from its closed form); the
    logical-zero state has parity +1 (reference tests/integration/
    test_utils_integration.py:290-300) and the unsupported forms raise."""
    from oracle import sfref

    try:
        sfref.import_strawberryfields()
    except ImportError:
        pytest.skip("reference sources not available")
    from strawberryfields.backends.fockbackend import FockBackend
    from strawberryfields_gb300 import FockGB300Backend

    dms = []
    for cls in (FockBackend, FockGB300Backend):
        b = cls()
        b.begin_circuit(2, cutoff_dim=D, pure=pure)
        b.displacement(0.3, 0.1, 0)
        b.prepare_gkp(state, eps, 1e-12, mode=1)
        dms.append(b.state().dm())
        if cls is FockGB300Backend:
            if state == [0, 0]:
                assert abs(b.state().parity_expectation([1]) - 1) < 1e-6
            with pytest.raises(NotImplementedError):
                b.prepare_gkp(state, eps, 1e-12, representation="complex", mode=0)
            with pytest.raises(NotImplementedError):
                b.prepare_gkp(state, eps, 1e-12, shape="hexagonal", mode=0)
    assert np.abs(dms[1] - dms[0]).max() < 1e-8


def test_program_with_new_and_del_runs_unchanged(cuda):
    """A program that creates and deletes modes (ops.New / ops.Del,
    strawberryfields/ops.py:2376,2423) gives the reference fock backend's
    state on fock_gb300."""
    pytest.importorskip("networkx")
    pytest.importorskip("sympy")
    from oracle import sfref

    try:
        sf = sfref.import_strawberryfields()
    except ImportError:
        pytest.skip("reference sources not available")
    from strawberryfields import ops as O
    from strawberryfields_gb300 import sf_backend

    prog = sf.Program(2)
    with prog.context as q:
        O.Sgate(0.25, 0.1) | q[0]
        O.Dgate(0.3, 0.4) | q[1]
        (c,) = O.New(1)
        O.BSgate(0.6, 0.2) | (q[1], c)
        O.Del | q[0]
        O.Kgate(0.07) | c
        O.S2gate(0.1, 0.3) | (q[1], c)
    states = []
    for backend in ("fock", sf_backend()):
        eng = sf.Engine(backend, backend_options={"cutoff_dim": 6})
        states.append(eng.run(prog).state.dm())
    assert states[1].shape == states[0].shape == (6,) * 4
    assert np.abs(states[1] - states[0]).max() < TOL


@pytest.mark.parametrize("pure", [True, False])
def test_homodyne_distribution_and_sample(cuda, pure):
    from strawberryfields_gb300.circuit import DeviceCircuit

    D = 10
    c = DeviceCircuit(2, D, pure=pure)
    c.squeeze(0.3, 0.7, 0)
    c.displacement(0.8, 0.4, 0)
    c.beamsplitter(0.6, 0.2, 0, 1)
    if not pure:
        c.loss(0.8, 0)
    rho = c.reduced_dm1(0).cpu().numpy()
    q, got = c.homodyne_pdf(0.9, 0, q_max=8, num_bins=4001)
    qr, ref = fo.homodyne_pdf(rho, 0.9, 2.0, 8, 4001)
    assert np.abs(got.cpu().numpy() - ref).max() < 1e-12
    # a sample, then mode 0 is in vacuum and the state normalised
    x = c.measure_homodyne(0.9, 0, rng=np.random.RandomState(5), num_bins=4001, max=8)
    assert x.shape == (1, 1) and -8 <= x[0, 0] <= 8
    marg = c.marginals().cpu().numpy()
    assert abs(marg[0, 0] - 1) < 1e-12 and abs(marg[1].sum() - 1) < 1e-12


def test_homodyne_coherent_state_moments(cuda):
    """|alpha> measured along phi = 0: mean sqrt(2 hbar) Re(alpha), variance hbar / 2."""
    from strawberryfields_gb300.circuit import DeviceCircuit

    c = DeviceCircuit(1, 20, pure=True)
    c.displacement(0.7, 0.3, 0)
    q, p = c.homodyne_pdf(0.0, 0, q_max=10, num_bins=20001)
    q, p = q.cpu().numpy(), p.cpu().numpy()
    mean = np.sum(q * p) / np.sum(p)
    var = np.sum(q * q * p) / np.sum(p) - mean ** 2
    assert abs(mean - 2 * 0.7 * np.cos(0.3)) < 1e-6
    assert abs(var - 1.0) < 1e-6


def _random_symplectic(m, seed):
    """A product of single-mode squeezers and rotations and beamsplitters
    (xxpp ordering)."""
    rng = np.random.default_rng(seed)

    def embed(Sk, modes):
        S = np.eye(2 * m)
        idx = list(modes) + [m + j for j in modes]
        S[np.ix_(idx, idx)] = Sk
        return S

    S = np.eye(2 * m)
    for j in range(m):
        r, ph, t = rng.uniform(0.1, 0.4), rng.uniform(0, 6), rng.uniform(0, 6)
        c, s = np.cosh(r), np.sinh(r)
        sq = np.array([[c - np.cos(ph) * s, -np.sin(ph) * s], [-np.sin(ph) * s, c + np.cos(ph) * s]])
        rt = np.array([[np.cos(t), -np.sin(t)], [np.sin(t), np.cos(t)]])
        S = embed(rt @ sq, [j]) @ S
    for j in range(m - 1):
        th, ph = rng.uniform(0, 1.5), rng.uniform(0, 6)
        ct, st, cp, sp = np.cos(th), np.sin(th), np.cos(ph), np.sin(ph)
        B = np.array([[ct, -cp * st, 0, -st * sp], [cp * st, ct, -st * sp, 0],
                      [0, st * sp, ct, -cp * st], [st * sp, 0, cp * st, ct]])
        S = embed(B, [j, j + 1]) @ S
    return S, rng.uniform(-0.4, 0.4, 2 * m)


@pytest.mark.parametrize("m,D", [(1, 9), (2, 6), (3, 4)])
def test_gaussian_gate_matrix_on_device(cuda, m, D):
    """The device Hermite recurrence against the oracle's (FP64, 1e-12)."""
    import ctypes

    import torch
    from strawberryfields_gb300 import _lib as L
    from strawberryfields_gb300 import gaussian

    S, d = _random_symplectic(m, 10 + m)
    R, y, C = gaussian.choi_parameters(S, d)
    mat = torch.empty([D] * (2 * m), dtype=torch.complex128, device="cuda")
    Rh = np.ascontiguousarray(R).view(np.float64)
    yh = np.ascontiguousarray(y).view(np.float64)
    Ch = np.array([C.real, C.imag])
    L.check(L.load().fock_gaussian_gate_matrix(m, D, Rh.ctypes.data, yh.ctypes.data, Ch.ctypes.data,
                                               mat.data_ptr(), None), "fock_gaussian_gate_matrix")
    ref = fo.gaussian_gate_matrix(S, d, D)
    assert np.abs(mat.cpu().numpy() - ref).max() < 1e-12
    assert ctypes is not None


@pytest.mark.parametrize("pure", [True, False])
@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_gaussian_gate_on_states(cuda, pure, dtype):
    """Ggate on modes (2, 0) of a 3-mode state after a few gates, against the
    oracle's dense apply (ket, or G rho G^dagger)."""
    D = 6
    b = make_backend(3, D, pure, dtype)
    b.squeeze(0.2, 0.3, 0)
    b.displacement(0.3, 1.0, 1)
    b.beamsplitter(0.5, 0.2, 0, 2)
    s0 = b.state()
    before = s0.ket() if pure else s0.dm()
    S, d = _random_symplectic(2, 3)
    b.gaussian_gate(S, d, 2, 0)
    got = b.state().ket() if pure else b.state().dm()
    G = fo.gaussian_gate_matrix(S, d, D)
    ref = fo.apply_gate_modes(before.astype(np.complex128), G, [2, 0], pure)
    tol = 1e-12 if dtype == "complex128" else 1e-5
    assert np.abs(got - ref).max() < tol
    with pytest.raises(ValueError, match="not symplectic"):
        b.gaussian_gate(S * 1.2, d, 2, 0)
