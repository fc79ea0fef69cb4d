"""GPU parity of the C-ABI kernels against the oracle (rows G1-G5, K1-K6, R1-R3).

Bars: complex128 states within 1e-12 (max abs) of the FP64 oracle, complex64
within 1e-5; gate matrices (always FP64) within 1e-12.
"""
import ctypes

import numpy as np
import pytest

from oracle import fock_oracle as fo
from tests.conftest import random_state

pytestmark = pytest.mark.gpu

TOL = {"complex128": 1e-12, "complex64": 1e-5}

ORACLE_1 = {3: fo.displacement, 4: fo.squeezing}
ORACLE_2 = {5: fo.beamsplitter, 6: fo.two_mode_squeeze, 7: fo.mzgate}


def _L():
    from strawberryfields_gb300 import _lib

    return _lib


def _stream():
    import torch

    return torch.cuda.current_stream().cuda_stream


def device_matrix(kind, p0, p1, D, deriv=False):
    import torch

    L = _L()
    lib = L.load()
    ne = lib.fock_gate_matrix_entries(kind, D)
    out = torch.empty(ne, dtype=torch.complex128, device="cuda")
    dout = torch.empty(ne, dtype=torch.complex128, device="cuda") if deriv else None
    ws = torch.empty(max(lib.fock_gate_workspace_bytes(kind, D), 16), dtype=torch.uint8, device="cuda")
    L.call("fock_gate_matrix", kind, p0, p1, D, out.data_ptr(), dout.data_ptr() if deriv else None,
           ws.data_ptr(), _stream())
    if kind in (5, 6, 7, 8, 9):
        dense = torch.empty(D ** 4, dtype=torch.complex128, device="cuda")
        L.call("fock_expand_blocks", kind, D, out.data_ptr(), dense.data_ptr(), _stream())
        res = dense.reshape(D, D, D, D).cpu().numpy()
        if deriv:
            dd = torch.empty(D ** 4, dtype=torch.complex128, device="cuda")
            L.call("fock_expand_blocks", kind, D, dout.data_ptr(), dd.data_ptr(), _stream())
            return res, dd.reshape(D, D, D, D).cpu().numpy()
        return res
    res = out.reshape(D, D).cpu().numpy()
    if deriv:
        return res, dout.reshape(D, D).cpu().numpy()
    return res


@pytest.mark.parametrize("D", [1, 2, 5, 12, 21])
@pytest.mark.parametrize("kind", [3, 4])
def test_single_mode_matrices(cuda, kind, D):
    r, phi = 0.37, 1.3
    M, dM = device_matrix(kind, r, phi, D, deriv=True)
    assert np.abs(M - ORACLE_1[kind](r, phi, D)).max() < 1e-12
    ref_d = fo.grad_displacement(r, phi, D)[0] if kind == 3 else fo.grad_squeezing(r, phi, D)[0]
    assert np.abs(dM - ref_d).max() < 1e-12


@pytest.mark.parametrize("D", [1, 2, 4, 7, 12])
@pytest.mark.parametrize("kind", [5, 6, 7])
def test_two_mode_matrices(cuda, kind, D):
    p0, p1 = 0.41, 2.2
    M, dM = device_matrix(kind, p0, p1, D, deriv=True)
    assert np.abs(M - ORACLE_2[kind](p0, p1, D)).max() < 1e-12
    if kind == 5:
        assert np.abs(dM - fo.grad_beamsplitter(p0, p1, D)[0]).max() < 1e-12
    elif kind == 6:
        assert np.abs(dM - fo.grad_two_mode_squeeze(p0, p1, D)[0]).max() < 1e-12
    else:
        h = 1e-6
        fd = (fo.mzgate(p0 + h, p1, D) - fo.mzgate(p0 - h, p1, D)) / (2 * h)
        assert np.abs(dM - fd).max() < 1e-8


@pytest.mark.parametrize("D", [3, 8])
def test_loss_superoperator(cuda, D):
    T = 0.83
    M = device_matrix(9, T, 0.0, D)  # [out_ket, in_ket, out_bra, in_bra]
    rho = np.random.default_rng(0).normal(size=(D, D)) + 0j
    out = np.einsum("anbm,nm->ab", M, rho)
    ref = sum(E @ rho @ E.conj().T for E in fo.loss_kraus(T, D))
    assert np.abs(out - ref).max() < 1e-12


# --------------------------------------------------------------------------
# gate application
# --------------------------------------------------------------------------

def gpu_apply(kind, p0, p1, m1, m2, state, N, D, pure, dtype, pre=None):
    import torch

    L = _L()
    lib = L.load()
    tdt = torch.complex128 if dtype == "complex128" else torch.complex64
    code = L.C128 if dtype == "complex128" else L.C64
    x = torch.as_tensor(state, device="cuda").to(tdt).contiguous()
    out = torch.empty_like(x)
    tmp = torch.empty_like(x)
    ws = torch.empty(max(lib.fock_gate_workspace_bytes(kind, D), 16), dtype=torch.uint8, device="cuda")
    pre_arr = None
    if pre is not None:
        pre_np = np.asarray(pre, dtype=np.float64)
        pre_arr = pre_np.ctypes.data_as(L._dp)
    L.call("fock_apply_gate", kind, float(p0), float(p1), m1, m2, N, D, int(pure), code, pre_arr,
           x.data_ptr(), out.data_ptr(), tmp.data_ptr(), ws.data_ptr(), _stream())
    return out.to(torch.complex128).cpu().numpy()


def oracle_apply(kind, p0, p1, m1, m2, state, N, D, pure, pre=None):
    s = np.array(state, dtype=np.complex128)
    if pre is not None:
        s = fo.apply_gate1(s, fo.phase(pre[0], D) @ fo.kerr(pre[1], D), m1, pure)
        if m2 >= 0 and kind in (5, 6, 7, 8):
            s = fo.apply_gate1(s, fo.phase(pre[2], D) @ fo.kerr(pre[3], D), m2, pure)
    if kind in ORACLE_1:
        return fo.apply_gate1(s, ORACLE_1[kind](p0, p1, D), m1, pure)
    if kind == 1:
        return fo.apply_gate1(s, fo.phase(p0, D), m1, pure)
    if kind == 2:
        return fo.apply_gate1(s, fo.kerr(p0, D), m1, pure)
    if kind == 8:
        return fo.apply_gate2(s, fo.cross_kerr(p0, D), m1, m2, pure)
    if kind == 9:
        return fo.apply_loss(s, p0, m1, N, pure)
    return fo.apply_gate2(s, ORACLE_2[kind](p0, p1, D), m1, m2, pure)


PAIRS = [(0, 1), (1, 0), (1, 2), (2, 1), (0, 2), (2, 0)]


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
@pytest.mark.parametrize("D", [5, 7])
@pytest.mark.parametrize("kind", [1, 2, 3, 4])
def test_apply_single_mode_pure(cuda, rng, kind, D, dtype):
    N = 3
    st = random_state(rng, (D,) * N)
    for m in range(N):
        got = gpu_apply(kind, 0.31, 0.7, m, -1, st, N, D, True, dtype)
        ref = oracle_apply(kind, 0.31, 0.7, m, -1, st, N, D, True)
        assert np.abs(got - ref).max() < TOL[dtype], (kind, m)


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
@pytest.mark.parametrize("D", [4, 6])
@pytest.mark.parametrize("kind", [5, 6, 7, 8])
def test_apply_two_mode_pure(cuda, rng, kind, D, dtype):
    N = 3
    st = random_state(rng, (D,) * N)
    for m1, m2 in PAIRS:
        got = gpu_apply(kind, 0.43, 1.9, m1, m2, st, N, D, True, dtype)
        ref = oracle_apply(kind, 0.43, 1.9, m1, m2, st, N, D, True)
        assert np.abs(got - ref).max() < TOL[dtype], (kind, m1, m2)


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
@pytest.mark.parametrize("kind", [1, 2, 3, 4, 9])
def test_apply_single_mode_mixed(cuda, rng, kind, dtype):
    N, D = 2, 5
    st = random_state(rng, (D,) * (2 * N), pure=False)
    for m in range(N):
        got = gpu_apply(kind, 0.83 if kind == 9 else 0.29, 0.4, m, -1, st, N, D, False, dtype)
        ref = oracle_apply(kind, 0.83 if kind == 9 else 0.29, 0.4, m, -1, st, N, D, False)
        assert np.abs(got - ref).max() < TOL[dtype], (kind, m)


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
@pytest.mark.parametrize("kind", [5, 6, 7, 8])
def test_apply_two_mode_mixed(cuda, rng, kind, dtype):
    N, D = 3, 4
    st = random_state(rng, (D,) * (2 * N), pure=False)
    for m1, m2 in PAIRS:
        got = gpu_apply(kind, 0.38, 0.9, m1, m2, st, N, D, False, dtype)
        ref = oracle_apply(kind, 0.38, 0.9, m1, m2, st, N, D, False)
        assert np.abs(got - ref).max() < TOL[dtype], (kind, m1, m2)


@pytest.mark.parametrize("pure", [True, False])
def test_pre_phases_fold(cuda, rng, pure):
    """Pending rotation/Kerr folded into the next gate equals applying them first."""
    N, D = 3, 5
    st = random_state(rng, (D,) * (N if pure else 2 * N), pure=pure)
    pre = [0.7, 0.05, -0.4, 0.02]
    for kind, m1, m2 in [(3, 1, -1), (4, 2, -1), (5, 0, 2), (6, 2, 1)]:
        p = pre if m2 >= 0 else pre[:2] + [0.0, 0.0]
        got = gpu_apply(kind, 0.3, 0.8, m1, m2, st, N, D, pure, "complex128", pre=p)
        ref = oracle_apply(kind, 0.3, 0.8, m1, m2, st, N, D, pure, pre=p)
        assert np.abs(got - ref).max() < 1e-12


def test_large_cutoff_generic_path(cuda, rng):
    """Block sizes beyond the unrolled range (D > 24) use the generic kernel."""
    N, D = 2, 27
    st = random_state(rng, (D,) * N)
    for kind, m1, m2 in [(3, 0, -1), (4, 1, -1), (5, 0, 1), (6, 1, 0)]:
        got = gpu_apply(kind, 0.2, 0.5, m1, m2, st, N, D, True, "complex128")
        ref = oracle_apply(kind, 0.2, 0.5, m1, m2, st, N, D, True)
        assert np.abs(got - ref).max() < 1e-11


# --------------------------------------------------------------------------
# other state ops and readouts
# --------------------------------------------------------------------------

def _t(x, dtype="complex128"):
    import torch

    return torch.as_tensor(x, device="cuda").to(torch.complex128 if dtype == "complex128" else torch.complex64)


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_mix_probs_marginals(cuda, rng, dtype):
    import torch

    L = _L()
    lib = L.load()
    N, D = 3, 6
    code = L.C128 if dtype == "complex128" else L.C64
    psi = random_state(rng, (D,) * N)
    x = _t(psi, dtype)
    dm = torch.empty([D] * (2 * N), dtype=x.dtype, device="cuda")
    L.call("fock_mix", N, D, code, x.data_ptr(), dm.data_ptr(), _stream())
    assert np.abs(dm.cpu().numpy() - fo.mix(psi, N)).max() < TOL[dtype]
    for pure, st in [(True, x), (False, dm)]:
        pr = torch.empty([D] * N, dtype=torch.float64, device="cuda")
        L.call("fock_probs", N, D, int(pure), code, st.data_ptr(), pr.data_ptr(), _stream())
        assert np.abs(pr.cpu().numpy() - fo.all_fock_probs(psi, N)).max() < TOL[dtype]
        mg = torch.empty((N, D), dtype=torch.float64, device="cuda")
        ws = torch.empty(lib.fock_marginals_workspace_bytes(N, D, int(pure), code), dtype=torch.uint8, device="cuda")
        L.call("fock_marginals", N, D, int(pure), code, st.data_ptr(), mg.data_ptr(), ws.data_ptr(), _stream())
        for m in range(N):
            assert np.abs(mg[m].cpu().numpy() - fo.marginal(psi, N, m)).max() < TOL[dtype]
        for m in range(N):
            rd = torch.empty((D, D), dtype=torch.complex128, device="cuda")
            ws = torch.empty(lib.fock_reduced_dm1_workspace_bytes(N, D, int(pure), code), dtype=torch.uint8,
                             device="cuda")
            L.call("fock_reduced_dm1", N, D, int(pure), code, m, st.data_ptr(), rd.data_ptr(), ws.data_ptr(),
                   _stream())
            assert np.abs(rd.cpu().numpy() - fo.reduced_dm(psi, N, m)).max() < TOL[dtype]


def test_vacuum_and_phases(cuda, rng):
    import torch

    L = _L()
    N, D = 3, 5
    v = torch.empty([D] * N, dtype=torch.complex128, device="cuda")
    L.call("fock_vacuum", N, D, 1, L.C128, v.data_ptr(), _stream())
    assert np.abs(v.cpu().numpy() - fo.vacuum(N, D)).max() == 0
    for pure in (True, False):
        st = random_state(rng, (D,) * (N if pure else 2 * N), pure=pure)
        ang = rng.normal(size=(N, D))
        x = _t(st)
        out = torch.empty_like(x)
        angd = torch.as_tensor(ang, device="cuda")
        ckm = (ctypes.c_int * 4)(0, 2, 1, 2)
        ckk = np.array([0.3, -0.2])
        L.call("fock_apply_phases", N, D, int(pure), L.C128, angd.data_ptr(), 2, ckm, ckk.ctypes.data_as(L._dp),
               x.data_ptr(), out.data_ptr(), _stream())
        ref = st.copy()
        for m in range(N):
            ref = fo.apply_gate1(ref, np.diag(np.exp(1j * ang[m])), m, pure)
        ref = fo.apply_gate2(ref, fo.cross_kerr(0.3, D), 0, 2, pure)
        ref = fo.apply_gate2(ref, fo.cross_kerr(-0.2, D), 1, 2, pure)
        assert np.abs(out.cpu().numpy() - ref).max() < 1e-12


def test_prepare_modes(cuda, rng):
    import torch

    L = _L()
    lib = L.load()
    N, D = 3, 4
    rho = random_state(rng, (D,) * (2 * N), pure=False)
    sub = random_state(rng, (D,) * 4, pure=False)  # two-mode mixed state
    for modes in ([2, 0], [1, 2]):
        x = _t(rho)
        out = torch.empty_like(x)
        ws = torch.empty(lib.fock_prepare_workspace_bytes(N, D, L.C128, 2), dtype=torch.uint8, device="cuda")
        mm = (ctypes.c_int * 2)(*modes)
        sd = _t(sub)
        L.call("fock_prepare_modes", N, D, L.C128, 2, mm, sd.data_ptr(), x.data_ptr(), out.data_ptr(),
               ws.data_ptr(), _stream())
        # oracle: trace out `modes`, tensor the sub state, move sub's modes into place
        rest = [m for m in range(N) if m not in modes]
        red = rho
        for m in sorted(modes, reverse=True):
            red = np.trace(red, axis1=2 * m, axis2=2 * m + 1)
        full = np.multiply.outer(red, sub)  # axes: rest (interleaved), then sub modes
        order = rest + list(modes)
        perm = [0] * (2 * N)
        for pos, m in enumerate(order):
            perm[2 * m] = 2 * pos
            perm[2 * m + 1] = 2 * pos + 1
        ref = np.transpose(full, perm)
        assert np.abs(out.cpu().numpy() - ref).max() < 1e-12


def test_invalid_arguments_raise(cuda):
    import torch

    L = _L()
    x = torch.zeros(16, dtype=torch.complex128, device="cuda")
    with pytest.raises(ValueError):
        L.call("fock_apply_gate", 3, 0.1, 0.0, 5, -1, 2, 4, 1, L.C128, None, x.data_ptr(), x.data_ptr(), None,
               x.data_ptr(), _stream())
    with pytest.raises(ValueError):
        L.call("fock_apply_gate", 42, 0.1, 0.0, 0, -1, 2, 4, 1, L.C128, None, x.data_ptr(), x.data_ptr(), None,
               x.data_ptr(), _stream())
