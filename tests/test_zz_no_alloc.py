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


def _largest_cutoff():
    """The entry point's cutoff limit, read from its own refusal message."""
    import re

    import torch
    from strawberryfields_gb300 import _lib as L

    x = torch.zeros(1, dtype=torch.complex128, device="cuda")
    out = torch.empty(1, dtype=torch.complex128, device="cuda")
    # the largest cutoff any kernel accepts (64) is refused on the scratch
    # size check, before the state or output is touched
    rc = L.load().fock_reduced_dm1_noalloc(1, 64, 1, L.C128, 0, x.data_ptr(), out.data_ptr(), None)
    assert rc == L.FOCK_ERR_INVALID
    msg = L.last_error()
    assert "too large" in msg
    return int(re.search(r"largest cutoff: (\d+)", msg).group(1))


def test_noalloc_large_state_and_limit(cuda):
    import torch
    from strawberryfields_gb300 import _lib as L

    rng = np.random.default_rng(5)
    # many column tiles: the grid is capped to the fixed number of slots
    st = random_state(rng, (12,) * 6)
    for _ in range(2):
        a = _rdm("noalloc", st, 6, 12, True, "complex64", 2)
        b = _rdm("workspace", st, 6, 12, True, "complex64", 2)
        assert np.abs(a - b).max() < 1e-5
    dmax = _largest_cutoff()
    assert dmax == 60  # FOCK_NOALLOC_MAX_CUTOFF in include/fock_gb300.h
    # the largest accepted cutoff (exactly the minimum number of slots)
    st = random_state(rng, (dmax,) * 2)
    for mode in (0, 1):
        a = _rdm("noalloc", st, 2, dmax, True, "complex128", mode)
        b = _rdm("workspace", st, 2, dmax, True, "complex128", mode)
        assert np.abs(a - b).max() < 1e-12
    # one past it is refused with a clear error
    x = torch.zeros(dmax + 1, dtype=torch.complex128, device="cuda")
    out = torch.empty((dmax + 1, dmax + 1), dtype=torch.complex128, device="cuda")
    rc = L.load().fock_reduced_dm1_noalloc(1, dmax + 1, 1, L.C128, 0, x.data_ptr(), out.data_ptr(), None)
    assert rc == L.FOCK_ERR_INVALID
    assert "too large" in L.last_error()


def test_noalloc_mixed_several_chunks(cuda):
    """A density matrix whose traced modes span several reduction chunks
    (D^(n-1) = 8192 traces: 2 chunks of 4096), checked twice in a row.  The
    entry point also caps the chunks at its scratch slots, but that cap cannot
    bind for a density matrix that fits in device memory (it needs
    D^(n-1) > 4096 * slots), so no test reaches it."""
    import torch
    from strawberryfields_gb300 import _lib as L

    N, D = 14, 2  # 2^28 complex64 entries (2.1 GB)
    g = torch.Generator(device="cuda").manual_seed(3)
    rho = torch.randn(D ** (2 * N), 2, device="cuda", generator=g, dtype=torch.float32)
    rho = torch.view_as_complex(rho).contiguous()
    lib = L.load()
    st = torch.cuda.current_stream().cuda_stream
    outs = []
    for mode in (0, N - 1):
        a = torch.empty((D, D), dtype=torch.complex128, device="cuda")
        b = torch.empty((D, D), dtype=torch.complex128, device="cuda")
        L.check(lib.fock_reduced_dm1_noalloc(N, D, 0, L.C64, mode, rho.data_ptr(), a.data_ptr(), st))
        ws = torch.empty(lib.fock_reduced_dm1_workspace_bytes(N, D, 0, L.C64), dtype=torch.uint8, device="cuda")
        L.check(lib.fock_reduced_dm1(N, D, 0, L.C64, mode, rho.data_ptr(), b.data_ptr(), ws.data_ptr(), st))
        scale = float(torch.abs(b).max())
        assert float(torch.abs(a - b).max()) <= 1e-5 * scale
        outs.append(a)
    assert float(torch.abs(outs[0] - outs[1]).max()) > 0  # different modes, different sums
