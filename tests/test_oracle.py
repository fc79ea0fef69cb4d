"""Pins of the CPU oracle (no GPU).

* gate matrices against scipy.linalg.expm of each generator (large cutoff,
  truncated) -- the restated thewalrus builders;
* the reference's analytic known answers (tests/backend in the reference);
* FP64 derivative matrices and the tape adjoint against central differences;
* the oracle's state updates against the reference's own Circuit (when the
  reference sources are present) and against the committed golden vectors.
"""
import math
import os

import numpy as np
import pytest
from scipy.linalg import expm

from oracle import fock_oracle as fo

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def a_op(D):
    return np.diag(np.sqrt(np.arange(1, D, dtype=float)), 1).astype(complex)


@pytest.mark.parametrize("r,phi", [(0.0, 0.0), (0.37, 1.1), (0.8, -2.3)])
def test_displacement_squeezing_vs_expm(r, phi):
    Db, D = 70, 12
    a = a_op(Db)
    ad = a.conj().T
    al = r * np.exp(1j * phi)
    assert np.abs(expm(al * ad - np.conj(al) * a)[:D, :D] - fo.displacement(r, phi, D)).max() < 1e-13
    Sm = expm(0.5 * (np.conj(al) * a @ a - al * ad @ ad))[:D, :D]
    assert np.abs(Sm - fo.squeezing(r, phi, D)).max() < 1e-13


@pytest.mark.parametrize("p0,p1", [(0.7, 1.3), (1.2, -0.4)])
def test_two_mode_gates_vs_expm(p0, p1):
    Db, D = 26, 7
    a = a_op(Db)
    I = np.eye(Db)
    a1, a2 = np.kron(a, I), np.kron(I, a)

    def sf_order(U):
        return U.reshape(Db, Db, Db, Db)[:D, :D, :D, :D].transpose(0, 2, 1, 3)

    B = expm(p0 * (np.exp(1j * p1) * a1 @ a2.conj().T - np.exp(-1j * p1) * a1.conj().T @ a2))
    assert np.abs(sf_order(B) - fo.beamsplitter(p0, p1, D)).max() < 1e-13
    r = p0 / 3
    z = r * np.exp(1j * p1)
    S2 = expm(z * a1.conj().T @ a2.conj().T - np.conj(z) * a1 @ a2)
    assert np.abs(sf_order(S2) - fo.two_mode_squeeze(r, p1, D)).max() < 1e-12
    R1 = lambda p: expm(1j * p * a1.conj().T @ a1)  # noqa: E731
    B50 = expm(np.pi / 4 * (np.exp(1j * np.pi / 2) * a1 @ a2.conj().T - np.exp(-1j * np.pi / 2) * a1.conj().T @ a2))
    MZ = B50 @ R1(p0) @ B50 @ R1(p1)
    assert np.abs(sf_order(MZ) - fo.mzgate(p0, p1, D)).max() < 1e-12


def test_known_answers():
    D = 12
    # coherent column (test_displacement_operation.py)
    al = 0.3 * np.exp(0.4j)
    k = np.arange(D)
    fac = np.array([math.factorial(int(i)) for i in k], dtype=float)
    coh = np.exp(-0.5 * abs(al) ** 2) * al ** k / np.sqrt(fac)
    assert np.abs(fo.displacement(abs(al), np.angle(al), D)[:, 0] - coh).max() < 1e-15
    # squeezed vacuum (Loudon 5.5.6)
    r, phi = 0.4, 0.9
    sv = np.zeros(D, dtype=complex)
    for n in range(0, D, 2):
        m = n // 2
        sv[n] = math.sqrt(math.factorial(2 * m)) / (2 ** m * math.factorial(m)) * (-np.exp(1j * phi) * np.tanh(r)) ** m
    assert np.abs(fo.squeezing(r, phi, D)[:, 0] - sv / math.sqrt(math.cosh(r))).max() < 1e-15
    # TMSV
    T = fo.two_mode_squeeze(r, phi, D)
    for n in range(D):
        assert abs(T[n, 0, n, 0] - (np.exp(1j * phi) * np.tanh(r)) ** n / np.cosh(r)) < 1e-15
    # beamsplitter on |alpha, 0> -> |t alpha, r alpha> (photon number < D exactly representable)
    th, ph = 0.6, 1.2
    psi = fo.apply_gate2(np.multiply.outer(fo.coherent_state(0.3, 0.0, D), fo.vacuum(1, D)), fo.beamsplitter(th, ph, D), 0, 1)
    ref = np.multiply.outer(fo.coherent_state(0.3 * np.cos(th), 0.0, D),
                            fo.coherent_state(0.3 * np.sin(th), ph, D))
    assert np.abs(psi - ref).max() < 1e-9
    # loss closed form against the Kraus sum
    rho = np.random.default_rng(0).normal(size=(D, D)) + 0j
    c = fo.loss_coeffs(0.8, D)
    out = np.zeros_like(rho)
    for n in range(D):
        for m in range(D):
            for l in range(min(n, m) + 1):
                out[n - l, m - l] += c[n, m, l] * rho[n, m]
    ref = sum(E @ rho @ E.conj().T for E in fo.loss_kraus(0.8, D))
    assert np.abs(out - ref).max() < 1e-14


def test_derivative_matrices_vs_central_differences():
    h = 1e-6
    for f, g, args in [(fo.displacement, fo.grad_displacement, (0.37, 1.1)),
                       (fo.squeezing, fo.grad_squeezing, (0.37, 1.1)),
                       (fo.beamsplitter, fo.grad_beamsplitter, (0.7, 1.1)),
                       (fo.two_mode_squeeze, fo.grad_two_mode_squeeze, (0.37, 1.1))]:
        d0, d1 = g(*args, 8)
        fd0 = (f(args[0] + h, args[1], 8) - f(args[0] - h, args[1], 8)) / (2 * h)
        fd1 = (f(args[0], args[1] + h, 8) - f(args[0], args[1] - h, 8)) / (2 * h)
        assert np.abs(d0 - fd0).max() < 1e-8 and np.abs(d1 - fd1).max() < 1e-8


def test_tape_adjoint_vs_central_differences():
    N, D = 3, 6
    gates = [(4, 0, -1, 0), (3, 1, -1, 2), (5, 0, 1, 4), (1, 2, -1, 6), (2, 1, -1, 7), (6, 1, 2, 8),
             (7, 0, 2, 10), (8, 0, 1, 12), (5, 2, 1, 13), (3, 2, -1, 15)]
    rng = np.random.default_rng(0)
    params = rng.uniform(0.05, 0.5, 17)
    t = rng.normal(size=(D,) * N) + 1j * rng.normal(size=(D,) * N)
    t /= np.linalg.norm(t)

    def loss(p):
        s = np.vdot(t, fo.run_gates(gates, p, N, D)[-1])
        return 1 - abs(s) ** 2

    s = np.vdot(t, fo.run_gates(gates, params, N, D)[-1])
    g = fo.adjoint_grads(gates, params, N, D, -2 * s * t)
    h = 1e-6
    fd = np.array([(loss(params + h * e) - loss(params - h * e)) / (2 * h) for e in np.eye(17)])
    assert np.abs(g - fd).max() < 1e-9


def _golden_cases():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def oracle_run(N, D, pure, ops):
    s = fo.vacuum(N, D, pure)
    for op in ops:
        name, rest = op[0], op[1:]
        if name == "S":
            s = fo.apply_gate1(s, fo.squeezing(rest[0], rest[1], D), rest[2], pure)
        elif name == "D":
            s = fo.apply_gate1(s, fo.displacement(rest[0], rest[1], D), rest[2], pure)
        elif name == "R":
            s = fo.apply_gate1(s, fo.phase(rest[0], D), rest[1], pure)
        elif name == "K":
            s = fo.apply_gate1(s, fo.kerr(rest[0], D), rest[1], pure)
        elif name == "BS":
            s = fo.apply_gate2(s, fo.beamsplitter(rest[0], rest[1], D), rest[2], rest[3], pure)
        elif name == "S2":
            s = fo.apply_gate2(s, fo.two_mode_squeeze(rest[0], rest[1], D), rest[2], rest[3], pure)
        elif name == "MZ":
            s = fo.apply_gate2(s, fo.mzgate(rest[0], rest[1], D), rest[2], rest[3], pure)
        elif name == "CK":
            s = fo.apply_gate2(s, fo.cross_kerr(rest[0], D), rest[1], rest[2], pure)
        elif name == "L":
            s = fo.apply_loss(s, rest[0], rest[1], N, pure)
            pure = False
        elif name == "MH":
            s = fo.homodyne_project(s, rest[0], rest[1], rest[2], N, pure)
    return s


@pytest.mark.parametrize("case", _golden_cases())
def test_oracle_reproduces_golden(case):
    from tests.golden.make_golden import decode

    z = np.load(os.path.join(GOLDEN, case + ".npz"))
    got = oracle_run(int(z["N"]), int(z["D"]), bool(z["pure"]), decode(z["ops"]))
    assert np.abs(got - z["state"]).max() < 1e-13


def test_oracle_vs_reference_circuit():
    """Regenerate one golden case through the reference Circuit directly."""
    from oracle import sfref

    if sfref.find_reference() is None:
        pytest.skip("reference sources not present")
    from tests.golden import make_golden as mg

    N, D, pure, ops = mg.pure_all(1)
    ref, _ = mg.run_reference(N, D, pure, ops)
    assert np.abs(oracle_run(N, D, pure, ops) - ref).max() < 1e-13


def test_oracle_mixed_gate_list_matches_golden():
    """The oracle's density-matrix gate-list runner reproduces the mixed golden
    vectors (unitaries on ket and bra axes, loss channels) of the reference
    Circuit."""
    import os

    from tests.gatelist import ops_to_gates
    from tests.golden.make_golden import decode

    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    n = 0
    for f in sorted(os.listdir(golden)):
        if not f.endswith(".npz"):
            continue
        z = np.load(os.path.join(golden, f))
        if bool(z["pure"]) or np.any(z["ops"][:, 0] == 10):  # gate lists only (10: homodyne)
            continue
        gates, params = ops_to_gates(decode(z["ops"]))
        rho = fo.run_gates_mixed(gates, params, int(z["N"]), int(z["D"]))
        assert np.abs(rho - z["state"]).max() < 1e-12, f
        n += 1
    assert n >= 2


def test_oracle_homodyne_pdf_coherent_state():
    """The restated homodyne distribution of |alpha> along phi: a normal
    distribution with mean sqrt(2 hbar) |alpha| cos(arg alpha - phi) and
    variance hbar / 2 (hbar = 2)."""
    D = 24
    psi = fo.coherent_state(0.8, 0.5, D)
    rho = np.outer(psi, psi.conj())
    for phi in (0.0, 0.9):
        q, p = fo.homodyne_pdf(rho, phi, 2.0, 10, 20001)
        mean = np.sum(q * p) / np.sum(p)
        var = np.sum(q * q * p) / np.sum(p) - mean ** 2
        assert abs(np.sum(p) - 1) < 1e-6
        assert abs(mean - 2 * 0.8 * np.cos(0.5 - phi)) < 1e-8
        assert abs(var - 1.0) < 1e-8


def _readout_cases():
    d = os.path.join(GOLDEN, "readouts")
    return sorted(f[:-4] for f in os.listdir(d) if f.endswith(".npz"))


@pytest.mark.parametrize("case", _readout_cases())
def test_oracle_wigner_reproduces_golden(case):
    """The oracle's Wigner iteration against the reference's own
    BaseFockState.wigner on the reduced states of a golden circuit."""
    r = np.load(os.path.join(GOLDEN, "readouts", case + ".npz"))
    z = np.load(os.path.join(GOLDEN, str(r["source"]) + ".npz"))
    N = int(z["N"])
    for i, m in enumerate(r["wigner_modes"]):
        rho = fo.reduced_dm(z["state"], N, int(m), bool(z["out_pure"]))
        W = fo.wigner(rho, r["xvec"], r["pvec"], float(r["hbar"]))
        assert np.abs(W - r["wigner"][i]).max() < 1e-14


def test_oracle_wigner_gaussian_known_answers():
    """Vacuum and coherent states: normal distributions with covariance
    hbar/2 and mean sqrt(2 hbar) (Re alpha, Im alpha) (the reference's
    tests/backend/test_states_wigner.py:55-110)."""
    from scipy.stats import multivariate_normal

    D, hbar = 30, 1.7
    xv = np.linspace(-4, 4, 33)
    X, P = np.meshgrid(xv, xv)
    grid = np.stack([X, P], axis=-1)
    for alpha in (0.0, 0.5 + 0.3j):
        psi = fo.coherent_state(abs(alpha), np.angle(alpha), D)
        W = fo.wigner(np.outer(psi, psi.conj()), xv, xv, hbar)
        mu = np.sqrt(2 * hbar) * np.array([alpha.real, alpha.imag])
        exact = multivariate_normal(mu, np.eye(2) * hbar / 2).pdf(grid)
        assert np.abs(W - exact).max() < 1e-12


class _HostState:
    """The readout host logic of FockStateGB300 on a numpy state, with the
    device reductions replaced by the oracle's (no GPU)."""

    def __init__(self, state, N, D, pure, hbar):
        from strawberryfields_gb300.states import FockStateGB300

        self.s = object.__new__(FockStateGB300)
        self.s._modes, self.s._cutoff, self.s._pure, self.s._hbar = N, D, pure, hbar
        self.state = state

        def reduced_dm(modes, **kwargs):
            modes = [modes] if isinstance(modes, int) else list(modes)
            if len(modes) == 1:
                return fo.reduced_dm(state, N, modes[0], pure)
            rho = state if not pure else fo.mix(state, N)
            for m in sorted(set(range(N)) - set(modes), reverse=True):
                rho = np.trace(rho, axis1=2 * m, axis2=2 * m + 1)
            return rho

        self.s.reduced_dm = reduced_dm


@pytest.mark.parametrize("case", _readout_cases())
def test_poly_quad_expectation_host_logic_matches_golden(case):
    r = np.load(os.path.join(GOLDEN, "readouts", case + ".npz"))
    z = np.load(os.path.join(GOLDEN, str(r["source"]) + ".npz"))
    h = _HostState(z["state"], int(z["N"]), int(z["D"]), bool(z["out_pure"]), float(r["hbar"]))
    for i in range(len(r["poly_k"])):
        A = None if r["poly_A_none"][i] else r["poly_A"][i]
        d = None if r["poly_d_none"][i] else r["poly_d"][i]
        got = h.s.poly_quad_expectation(A, d, float(r["poly_k"][i]), phi=float(r["poly_phi"][i]))
        assert np.allclose(got, r["poly_mean_var"][i], rtol=1e-12, atol=1e-12), (case, i)


def test_poly_quad_expectation_argument_checks():
    h = _HostState(fo.vacuum(2, 4), 2, 4, True, 2.0)
    with pytest.raises(ValueError, match="2Nx2N"):
        h.s.poly_quad_expectation(np.eye(3))
    with pytest.raises(ValueError, match="symmetric"):
        h.s.poly_quad_expectation(np.triu(np.ones((4, 4))))
    with pytest.raises(ValueError, match="length 2N"):
        h.s.poly_quad_expectation(np.eye(4), np.ones(3))
    assert h.s.poly_quad_expectation(None, None, 2.5) == (2.5, 0.0)


def _symplectics():
    """thewalrus-convention symplectic matrices (xxpp) of the SF gates."""
    def sq(r, phi):
        c, s = np.cosh(r), np.sinh(r)
        return np.array([[c - np.cos(phi) * s, -np.sin(phi) * s], [-np.sin(phi) * s, c + np.cos(phi) * s]])

    def rot(t):
        return np.array([[np.cos(t), -np.sin(t)], [np.sin(t), np.cos(t)]])

    def bs(th, ph):
        ct, st, cp, sp = np.cos(th), np.sin(th), np.cos(ph), np.sin(ph)
        return np.array([[ct, -cp * st, 0, -st * sp], [cp * st, ct, -st * sp, 0],
                         [0, st * sp, ct, -cp * st], [st * sp, 0, cp * st, ct]])

    def s2(r, ph):
        ch, sh, cp, sp = np.cosh(r), np.sinh(r), np.cos(ph), np.sin(ph)
        return np.array([[ch, cp * sh, 0, sp * sh], [cp * sh, ch, sp * sh, 0],
                         [0, sp * sh, ch, -cp * sh], [sp * sh, 0, -cp * sh, ch]])

    return sq, rot, bs, s2


def test_gaussian_gate_matrix_is_the_exact_gate():
    """The Ggate restatement (choi_trick + renormalised Hermite recurrence)
    reproduces the exact truncated matrices of the squeezer, displacement,
    rotation, beamsplitter and two-mode squeezer (themselves pinned to expm):
    this fixes its conventions (xxpp symplectic, d = (x, p) with hbar 2,
    output indices first)."""
    sq, rot, bs, s2 = _symplectics()
    D = 7
    G = fo.gaussian_gate_matrix(sq(0.4, 0.7), np.zeros(2), D)
    assert np.abs(G - fo.squeezing(0.4, 0.7, D)).max() < 1e-13
    al = 0.3 * np.exp(0.5j)
    G = fo.gaussian_gate_matrix(np.eye(2), [2 * al.real, 2 * al.imag], D)
    assert np.abs(G - fo.displacement(0.3, 0.5, D)).max() < 1e-13
    assert np.abs(fo.gaussian_gate_matrix(rot(0.6), np.zeros(2), D) - fo.phase(0.6, D)).max() < 1e-13
    D = 6
    G = fo.gaussian_gate_matrix(bs(0.7, 0.4), np.zeros(4), D)
    assert np.abs(G.transpose(0, 2, 1, 3) - fo.beamsplitter(0.7, 0.4, D)).max() < 1e-13
    G = fo.gaussian_gate_matrix(s2(0.3, 1.1), np.zeros(4), D)
    assert np.abs(G.transpose(0, 2, 1, 3) - fo.two_mode_squeeze(0.3, 1.1, D)).max() < 1e-13


def test_gaussian_host_choi_matches_oracle():
    from strawberryfields_gb300 import gaussian

    sq, rot, bs, s2 = _symplectics()
    S = bs(0.3, 0.9) @ np.kron(np.eye(2), np.eye(2))
    d = np.array([0.2, -0.1, 0.3, 0.05])
    R1, y1, C1 = gaussian.choi_parameters(S, d)
    R2, y2, C2 = fo._choi(S, d)
    assert np.abs(R1 - R2).max() < 1e-14 and np.abs(y1 - y2).max() < 1e-14 and abs(C1 - C2) < 1e-14
    assert gaussian.is_symplectic(S) and not gaussian.is_symplectic(S * 1.1)
    with pytest.raises(ValueError, match="not symplectic"):
        gaussian.check_gate(S * 1.1, d)
    with pytest.raises(ValueError, match="compatible"):
        gaussian.check_gate(S, d[:2])


def test_gaussian_choi_parameters_of_the_identity_and_a_displacement():
    """S = I, d = 0 is the identity gate: R couples each output index to its
    input index only (R = [[0, -I], [-I, 0]], so the Hermite tensor is
    delta(out, in)), y = 0, C = 1.  A pure displacement keeps that R and
    gives y = (alpha, -conj(alpha)), C = exp(-|alpha|^2 / 2) = <0|D(alpha)|0>."""
    from strawberryfields_gb300 import gaussian

    for m in (1, 2, 3):
        R, y, C = gaussian.choi_parameters(np.eye(2 * m), np.zeros(2 * m))
        R_id = -np.block([[np.zeros((m, m)), np.eye(m)], [np.eye(m), np.zeros((m, m))]])
        assert np.abs(R - R_id).max() < 1e-14 and np.abs(y).max() < 1e-14 and abs(C - 1) < 1e-14
    d = np.array([0.4, -0.2, 0.6, 0.1])  # (x1, x2, p1, p2): alpha = (x + i p) / 2
    R, y, C = gaussian.choi_parameters(np.eye(4), d)
    alpha = (d[:2] + 1j * d[2:]) / 2
    assert np.abs(R + np.block([[np.zeros((2, 2)), np.eye(2)], [np.eye(2), np.zeros((2, 2))]])).max() < 1e-14
    assert np.abs(y[:2] - alpha).max() < 1e-14 and np.abs(y[2:] + alpha.conj()).max() < 1e-14
    assert abs(C - np.exp(-0.5 * np.sum(np.abs(alpha) ** 2))) < 1e-14
