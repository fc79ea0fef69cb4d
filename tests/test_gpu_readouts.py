"""Phase-space readouts of the GPU state object against the reference's own
BaseFockState outputs (golden vectors in tests/golden/readouts, made by
tests/golden/make_readouts.py) and the oracle's restatement of its Wigner
iteration.  complex128 states: 1e-13 absolute on W (|W| <= 1/(pi hbar));
complex64 states: 1e-6.
"""
import os

import numpy as np
import pytest

from oracle import fock_oracle as fo

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(f[:-4] for f in os.listdir(os.path.join(GOLDEN, "readouts")) if f.endswith(".npz"))


def _state(case, dtype="complex128"):
    import torch
    from strawberryfields_gb300.states import FockStateGB300

    r = np.load(os.path.join(GOLDEN, "readouts", case + ".npz"))
    z = np.load(os.path.join(GOLDEN, str(r["source"]) + ".npz"))
    t = torch.as_tensor(z["state"], device="cuda").to(getattr(torch, dtype))
    st = FockStateGB300(t, int(z["N"]), bool(z["out_pure"]), int(z["D"]), hbar=float(r["hbar"]))
    return st, r, z


@pytest.mark.parametrize("case", CASES)
def test_wigner_and_quadrature_values_match_reference(cuda, case):
    st, r, _ = _state(case)
    for i, m in enumerate(r["wigner_modes"]):
        W = st.wigner(int(m), r["xvec"], r["pvec"])
        assert W.shape == (len(r["pvec"]), len(r["xvec"]))
        assert np.abs(W - r["wigner"][i]).max() < 1e-13
    assert np.abs(st.x_quad_values(0, r["xvec"], r["pvec"]) - r["x_quad"]).max() < 1e-13
    assert np.abs(st.p_quad_values(0, r["xvec"], r["pvec"]) - r["p_quad"]).max() < 1e-13


@pytest.mark.parametrize("case", CASES)
def test_poly_quad_expectation_matches_reference(cuda, case):
    st, r, _ = _state(case)
    for i in range(len(r["poly_k"])):
        A = None if r["poly_A_none"][i] else r["poly_A"][i]
        d = None if r["poly_d_none"][i] else r["poly_d"][i]
        got = st.poly_quad_expectation(A, d, float(r["poly_k"][i]), phi=float(r["poly_phi"][i]))
        assert np.allclose(got, r["poly_mean_var"][i], rtol=1e-12, atol=1e-12), (case, i)


@pytest.mark.parametrize("case", CASES)
def test_quad_expectation_matches_reference(cuda, case):
    st, r, z = _state(case)
    for m in range(int(z["N"])):
        for i, phi in enumerate(r["quad_phis"]):
            got = st.quad_expectation(m, phi=float(phi))
            assert np.allclose(got, r["quad_mean_var"][m, i], rtol=1e-12, atol=1e-12), (case, m, phi)


def test_wigner_complex64_state(cuda):
    st, r, _ = _state(CASES[0], "complex64")
    W = st.wigner(0, r["xvec"], r["pvec"])
    assert np.abs(W - r["wigner"][0]).max() < 1e-6


def _device_wigner(rho, xv, pv, hbar):
    import torch
    from strawberryfields_gb300 import _lib as L

    rt = torch.as_tensor(rho, device="cuda")
    xt = torch.as_tensor(np.asarray(xv, dtype=np.float64), device="cuda")
    pt = torch.as_tensor(np.asarray(pv, dtype=np.float64), device="cuda")
    out = torch.empty((len(pv), len(xv)), dtype=torch.float64, device="cuda")
    L.call("fock_wigner", rho.shape[0], rt.data_ptr(), xt.data_ptr(), len(xv), pt.data_ptr(), len(pv), hbar,
           out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    return out.cpu().numpy()


@pytest.mark.parametrize("D,n", [(1, 5), (20, 120)])
def test_wigner_kernel_vs_oracle(cuda, D, n):
    """Random density matrices on ragged grids against the reference's
    iteration, in the range where it keeps its digits (|x|, |p| <= 3 at
    cutoff 20; it loses 4e-13 at cutoff 30 and 5e-8 at cutoff 64 there)."""
    rng = np.random.default_rng(D)
    Z = rng.normal(size=(D, D)) + 1j * rng.normal(size=(D, D))
    rho = Z @ Z.conj().T
    rho /= np.trace(rho)
    xv = np.linspace(-3, 3, n)
    pv = np.linspace(-2.5, 3, n + 3)
    want = fo.wigner(rho, xv, pv, 1.3)
    assert np.abs(_device_wigner(rho, xv, pv, 1.3) - want).max() < 1e-12


def test_wigner_kernel_wide_range_vs_high_precision(cuda):
    """Cutoffs 30 and 64 (the staged tables then exceed the default 48 KB of
    shared memory) out to |x| = 9: far from the origin the Wigner sum cancels
    large terms (the reference's double-precision iteration is off by up to
    4e-7 there); the device values agree with 50-digit evaluations
    (tests/golden/make_wigner_highprec.py) to 1e-13."""
    z = np.load(os.path.join(GOLDEN, "highprec", "wigner.npz"))
    for D in (30, 64):
        got = _device_wigner(z[f"rho{D}"], z[f"x{D}"], z[f"p{D}"], float(z["hbar"]))
        assert np.abs(got - z[f"w{D}"]).max() < 1e-13, D


def test_wigner_empty_grid_and_bad_arguments(cuda):
    import torch
    from strawberryfields_gb300 import _lib as L

    st, r, _ = _state(CASES[0])
    assert st.wigner(0, [], r["pvec"]).shape == (len(r["pvec"]), 0)
    rho = torch.eye(4, dtype=torch.complex128, device="cuda")
    x = torch.zeros(3, dtype=torch.float64, device="cuda")
    out = torch.empty(9, dtype=torch.float64, device="cuda")
    lib = L.load()
    assert lib.fock_wigner(0, rho.data_ptr(), x.data_ptr(), 3, x.data_ptr(), 3, 2.0, out.data_ptr(), None) \
        == L.FOCK_ERR_INVALID
    assert lib.fock_wigner(4, rho.data_ptr(), x.data_ptr(), 3, x.data_ptr(), 3, 0.0, out.data_ptr(), None) \
        == L.FOCK_ERR_INVALID


def test_state_equality(cuda):
    """BaseFockState.__eq__ (states.py:503): density matrices within 1e-10."""
    import torch
    from strawberryfields_gb300.states import FockStateGB300

    a, _, z = _state(CASES[0])
    b = FockStateGB300(torch.as_tensor(z["state"], device="cuda") * np.exp(0.3j), int(z["N"]), True, int(z["D"]))
    c = FockStateGB300(torch.as_tensor(z["state"], device="cuda") * 1.001, int(z["N"]), True, int(z["D"]))
    assert a == b  # a global phase leaves the density matrix unchanged
    assert not (a == c)
    assert not (a == "state")
