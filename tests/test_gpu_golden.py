"""The GPU backend reproduces the golden vectors generated by the reference's
own fockbackend Circuit (tests/golden/make_golden.py) within 1e-12 (complex128)
and 1e-5 (complex64)."""
import os

import numpy as np
import pytest

from tests.golden.make_golden import decode

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def run_backend(N, D, pure, ops, dtype):
    from strawberryfields_gb300 import FockGB300Backend

    b = FockGB300Backend()
    b.begin_circuit(N, cutoff_dim=D, pure=pure, dtype=dtype)
    table = {"S": b.squeeze, "D": b.displacement, "R": b.rotation, "K": b.kerr_interaction, "BS": b.beamsplitter,
             "S2": b.two_mode_squeeze, "MZ": b.mzgate, "CK": b.cross_kerr_interaction, "L": b.loss,
             "MH": lambda phi, x, m: b.measure_homodyne(phi, m, select=x)}
    for op in ops:
        table[op[0]](*op[1:])
    st = b.state()
    return st.ket() if st.is_pure else st.dm(), st.is_pure


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
@pytest.mark.parametrize("case", CASES)
def test_backend_reproduces_golden(cuda, case, dtype):
    z = np.load(os.path.join(GOLDEN, case + ".npz"))
    got, is_pure = run_backend(int(z["N"]), int(z["D"]), bool(z["pure"]), decode(z["ops"]), dtype)
    assert is_pure == bool(z["out_pure"])
    tol = 1e-12 if dtype == "complex128" else 1e-5
    assert np.abs(got.astype(np.complex128) - z["state"]).max() < tol


def test_compiled_circuit_reproduces_golden_cfg1(cuda):
    """The fused compiled path on the 3-mode cutoff-10 plain circuit."""
    import torch
    from strawberryfields_gb300 import CompiledCircuit

    kinds = {"S": 4, "D": 3, "BS": 5, "R": 1, "K": 2}
    for case in [c for c in CASES if c.startswith("cfg1")]:
        z = np.load(os.path.join(GOLDEN, case + ".npz"))
        gates, params = [], []
        for op in decode(z["ops"]):
            name, rest = op[0], op[1:]
            npar = 2 if name in ("S", "D", "BS") else 1
            modes = rest[npar:]
            gates.append((kinds[name], modes[0], modes[1] if len(modes) > 1 else -1, len(params)))
            params += list(rest[:npar])
        circ = CompiledCircuit(3, 10, gates, len(params), dtype=torch.complex128)
        psi = circ(torch.tensor(params, device="cuda"))
        assert np.abs(psi.cpu().numpy() - z["state"]).max() < 1e-12
