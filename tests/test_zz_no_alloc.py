"""fock_reduced_dm1_noalloc: the reduced density matrix for callers that cannot
allocate device memory (its partial sums live in a fixed array inside the
library).  Checked through the C ABI against fock_reduced_dm1, which uses a
caller-provided workspace, on two calls in a row (the fixed array keeps the
previous call's contents).  Collected last so a failure here cannot hide
another test's result."""
import ctypes

import numpy as np
import pytest

from tests.conftest import random_state

pytestmark = pytest.mark.gpu


def _rdm(fn, state, N, D, pure, dtype, mode):
    import torch
    from strawberryfields_gb300 import _lib as L

    lib = L.load()
    code = L.C128 if dtype == "complex128" else L.C64
    x = torch.as_tensor(state, device="cuda").to(torch.complex128 if dtype == "complex128" else torch.complex64)
    out = torch.empty((D, D), dtype=torch.complex128, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    if fn == "noalloc":
        L.check(lib.fock_reduced_dm1_noalloc(N, D, int(pure), code, mode, x.data_ptr(), out.data_ptr(), st))
    else:
        ws = torch.empty(lib.fock_reduced_dm1_workspace_bytes(N, D, int(pure), code), dtype=torch.uint8,
                         device="cuda")
        L.check(lib.fock_reduced_dm1(N, D, int(pure), code, mode, x.data_ptr(), out.data_ptr(), ws.data_ptr(), st))
    return out.cpu().numpy()


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
@pytest.mark.parametrize("pure", [True, False])
def test_noalloc_matches_workspace_entry_point(cuda, pure, dtype):
    rng = np.random.default_rng(99)
    tol = 1e-12 if dtype == "complex128" else 1e-5
    N, D = (4, 9) if pure else (3, 5)
    # two calls in a row with different states and modes
    for call, mode in enumerate([1, N - 1]):
        st = random_state(rng, (D,) * (N if pure else 2 * N), pure=pure)
        a = _rdm("noalloc", st, N, D, pure, dtype, mode)
        b = _rdm("workspace", st, N, D, pure, dtype, mode)
        assert np.abs(a - b).max() < tol, (call, np.abs(a - b).max())


def test_noalloc_large_state_and_limit(cuda):
    from strawberryfields_gb300 import _lib as L

    rng = np.random.default_rng(5)
    # many column tiles: the grid is capped to the fixed number of slots
    st = random_state(rng, (12,) * 6)
    for _ in range(2):
        a = _rdm("noalloc", st, 6, 12, True, "complex64", 2)
        b = _rdm("workspace", st, 6, 12, True, "complex64", 2)
        assert np.abs(a - b).max() < 1e-5
    # cutoff beyond the fixed scratch is refused with a clear error
    import torch

    x = torch.zeros(61, dtype=torch.complex128, device="cuda")
    out = torch.empty((61, 61), dtype=torch.complex128, device="cuda")
    rc = L.load().fock_reduced_dm1_noalloc(1, 61, 1, L.C128, 0, x.data_ptr(), out.data_ptr(), None)
    assert rc == L.FOCK_ERR_INVALID
    assert "too large" in L.last_error()
