"""The C-ABI library without a GPU: it builds, loads, exports every symbol the
header declares, validates arguments before touching the device, and its
host-side circuit compiler (gate fusion) behaves as documented."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fock_gb300.h")


@pytest.fixture(scope="module")
def lib():
    from strawberryfields_gb300 import _lib
    from strawberryfields_gb300 import build as b

    if not os.path.exists(_lib.LIBPATH):
        b.build()
    return _lib.load()


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fock_[a-z0-9_]+)\s*\(", src)))


def test_header_and_binding_agree():
    from strawberryfields_gb300 import _lib

    assert declared_functions() == _lib.exported_symbols()


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_size_queries(lib):
    from oracle import fock_oracle as fo  # noqa: F401  (checker import only)

    assert lib.fock_gate_matrix_entries(3, 12) == 144
    assert lib.fock_gate_matrix_entries(5, 12) == 12 * (2 * 144 + 1) // 3
    assert lib.fock_gate_matrix_entries(6, 4) == sum(min(k, 8 - k) ** 2 for k in range(1, 8))
    assert lib.fock_gate_matrix_entries(42, 12) == 0
    assert lib.fock_gate_matrix_entries(3, 0) == 0
    assert lib.fock_gate_workspace_bytes(4, 10) > 2 * 100 * 16


def test_invalid_arguments_rejected_on_host(lib):
    from strawberryfields_gb300 import _lib

    dummy = ctypes.c_void_p(16)
    # unknown kind, bad mode, bad cutoff, bad dtype, in == out: all caught before any CUDA call
    cases = [
        (42, 0, -1, 2, 4, 1, 0),
        (3, 5, -1, 2, 4, 1, 0),
        (3, 0, -1, 2, 0, 1, 0),
        (3, 0, -1, 2, 4, 1, 7),
        (5, 0, 0, 2, 4, 1, 0),
    ]
    for kind, m1, m2, n, D, pure, dt in cases:
        rc = lib.fock_apply_gate(kind, 0.1, 0.0, m1, m2, n, D, pure, dt, None, dummy, ctypes.c_void_p(32), None,
                                 dummy, None)
        assert rc == _lib.FOCK_ERR_INVALID
        assert _lib.last_error()
    rc = lib.fock_apply_gate(3, 0.1, 0.0, 0, -1, 2, 4, 1, 0, None, dummy, dummy, None, dummy, None)
    assert rc == _lib.FOCK_ERR_INVALID and "distinct" in _lib.last_error()
    # loss on a pure state is refused (the host mixes first)
    rc = lib.fock_apply_gate(9, 0.5, 0.0, 0, -1, 2, 4, 1, 0, None, dummy, ctypes.c_void_p(32), None, dummy, None)
    assert rc == _lib.FOCK_ERR_INVALID and "mixed" in _lib.last_error()
    with pytest.raises(ValueError):
        _lib.check(rc)


def _plan(gates, n_params, N=3, D=6, pure=1, dtype=0):
    from strawberryfields_gb300 import _lib

    lib = _lib.load()
    arr = (_lib.FockGate * max(len(gates), 1))()
    for i, (k, a, b, p) in enumerate(gates):
        arr[i].kind, arr[i].mode1, arr[i].mode2, arr[i].pidx = k, a, b, p
    plan = ctypes.c_void_p()
    rc = lib.fock_plan_create(N, D, pure, dtype, arr, len(gates), n_params, ctypes.byref(plan))
    return rc, plan


def _ops(plan):
    from strawberryfields_gb300 import _lib

    lib = _lib.load()
    info = _lib.PlanInfo()
    assert lib.fock_plan_get_info(plan, ctypes.byref(info)) == 0
    out = []
    for k in range(info.n_ops):
        a, b, c, d = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        assert lib.fock_plan_op(plan, k, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d)) == 0
        out.append((a.value, b.value, c.value, d.value))
    return info, out


def test_plan_fuses_diagonal_gates(lib):
    """Rotation/Kerr/cross-Kerr never get their own pass when a neighbour exists."""
    from strawberryfields_gb300.qnn import qnn_gates

    gates, npar = qnn_gates(6, 4)
    rc, plan = _plan(gates, npar, N=6, D=12)
    assert rc == 0
    info, ops = _ops(plan)
    nondiag = [g for g in gates if g[0] not in (1, 2, 8)]
    assert info.n_ops == len(nondiag) == 168
    assert sum(o[3] for o in ops) == len(gates)  # every gate accounted for once
    assert info.state_bytes == 12 ** 6 * 8
    assert info.bytes_fwd == 2 * info.state_bytes * 168
    lib.fock_plan_destroy(plan)


def test_plan_fusion_edge_cases(lib):
    # R on a mode no other gate touches -> its own identity op; CK not followed
    # by a gate on its pair -> its own op; trailing K -> output term of the last op
    gates = [(1, 2, -1, 0), (5, 0, 1, 1), (8, 0, 1, 3), (2, 0, -1, 4), (4, 1, -1, 5)]
    rc, plan = _plan(gates, 7)
    assert rc == 0
    info, ops = _ops(plan)
    kinds = [(o[0], o[1], o[2]) for o in ops]
    assert (2, 0, 1) in kinds          # BS (number-sum blocks)
    assert (1, 1, -1) in kinds         # squeezer (dense)
    assert (2, 0, 1) in kinds[1:] or sum(1 for k in kinds if k == (2, 0, 1)) == 2  # CK identity op
    assert (1, 2, -1) in kinds         # identity op carrying R on mode 2
    assert sum(o[3] for o in ops) == len(gates)
    lib.fock_plan_destroy(plan)


def test_plan_rejects_bad_gate_lists(lib):
    from strawberryfields_gb300 import _lib

    for gates, npar in [([(3, 4, -1, 0)], 2), ([(5, 0, 0, 0)], 2), ([(3, 0, -1, 1)], 2), ([(42, 0, -1, 0)], 2)]:
        rc, plan = _plan(gates, npar)
        assert rc == _lib.FOCK_ERR_INVALID
    # a loss channel needs a density matrix
    rc, plan = _plan([(9, 0, -1, 0)], 1)
    assert rc == _lib.FOCK_ERR_UNSUPPORTED


def test_mixed_plan_structure(lib):
    """Density-matrix plans: each unitary op runs on the ket axes and, with the
    conjugate matrix, on the bra axes; a loss channel is one superoperator op;
    phases next to a loss are carried by it."""
    # S(0), BS(0,1), K(1), loss(1), R(0)
    gates = [(4, 0, -1, 0), (5, 0, 1, 2), (2, 1, -1, 4), (9, 1, -1, 5), (1, 0, -1, 6)]
    rc, plan = _plan(gates, 7, pure=0)
    assert rc == 0
    info, ops = _ops(plan)
    kinds = [(o[0], o[1], o[2]) for o in ops]
    assert kinds == [(1, 0, -1), (1, 0, -1), (2, 0, 1), (2, 0, 1), (3, 1, -1)]
    # every gate accounted for once (bra-side ops carry no fused count); the
    # trailing rotation on mode 0 rides on the beamsplitter's ket op
    assert sum(o[3] for o in ops) == len(gates)
    assert info.state_elems == 6 ** 6 and info.n_ops == 5  # 3 modes, D = 6, density matrix
    lib.fock_plan_destroy(plan)


def test_plan_tune_knobs(lib):
    """fock_plan_tune: per-op kernel family and adjoint CTA density, argument
    checks, and the workspace it implies (more adjoint CTAs, more partials)."""
    from strawberryfields_gb300 import _lib
    from strawberryfields_gb300.qnn import qnn_gates

    gates, npar = qnn_gates(6, 1)
    rc, plan = _plan(gates, npar, N=6, D=10)
    assert rc == 0
    info, ops = _ops(plan)

    def cfg(k):
        f, c, ok, tc = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        assert lib.fock_plan_op_config(plan, k, ctypes.byref(f), ctypes.byref(c), ctypes.byref(ok),
                                       ctypes.byref(tc)) == 0
        return f.value, c.value, ok.value, tc.value

    configs = [cfg(k) for k in range(info.n_ops)]
    assert all(c == 8 for _, c, _, _ in configs)
    assert any(ok for _, _, ok, _ in configs)
    two = [k for k, o in enumerate(ops) if o[0] == 2 and configs[k][2]]
    assert two and all(configs[k][3] == 32 for k in two)
    assert lib.fock_plan_tune(plan, 0, 2, 0, 0) == _lib.FOCK_ERR_INVALID
    assert lib.fock_plan_tune(plan, 0, -1, 65, 0) == _lib.FOCK_ERR_INVALID
    assert lib.fock_plan_tune(plan, 0, -1, 0, 40) == _lib.FOCK_ERR_INVALID
    assert lib.fock_plan_tune(plan, info.n_ops, -1, 4, 0) == _lib.FOCK_ERR_INVALID
    ws0 = info.workspace_bytes
    sizes = []
    for ctas in (2, 16):
        for k in range(info.n_ops):
            assert lib.fock_plan_tune(plan, k, 0, ctas, 0) == 0
        sizes.append(_ops(plan)[0].workspace_bytes)
    assert sizes[1] > sizes[0] and cfg(0)[:2] == (0, 16)
    # plane tiles of 24 columns on a two-mode op (its plane partial sums follow its grid)
    assert lib.fock_plan_tune(plan, two[0], 1, 0, 24) == 0 and cfg(two[0])[3] == 24
    for k in range(info.n_ops):
        assert lib.fock_plan_tune(plan, k, configs[k][0], configs[k][1], configs[k][3] if configs[k][3] <= 32 else 0) == 0
    assert _ops(plan)[0].workspace_bytes == ws0 and cfg(two[0])[3] == 32
    lib.fock_plan_destroy(plan)
    # two-mode plane tiles stop at cutoff 16: a cutoff-18 beamsplitter has none
    rc, plan = _plan([(5, 0, 1, 0)], 2, N=2, D=18)
    assert rc == 0 and lib.fock_plan_tune(plan, 0, 1, 0, 0) == _lib.FOCK_ERR_UNSUPPORTED
    lib.fock_plan_destroy(plan)


def test_product_path_has_no_cpu_fallback():
    """The package never imports the oracle."""
    pkg = os.path.join(ROOT, "strawberryfields_gb300")
    for fn in os.listdir(pkg):
        if fn.endswith(".py"):
            src = open(os.path.join(pkg, fn)).read()
            assert "oracle" not in re.sub(r"#.*|\"\"\"[\s\S]*?\"\"\"", "", src), fn


def test_autotune_selection_logic(monkeypatch):
    """CompiledCircuit.autotune's choice, with the device replaced by a cost
    model (no GPU): per op the cheapest candidate, then the whole-step check
    that falls back to the starting CTA densities when the per-op picks lose
    on the whole step."""
    import types

    from strawberryfields_gb300 import autograd

    class FakeLib:
        def fock_plan_enable_timing(self, plan, on):
            return 0

    monkeypatch.setattr(autograd.L, "load", lambda: FakeLib())

    # op 0: dense, no plane kernel; op 1: two-mode, plane by default; op 2: two-mode on block kernels
    start = [(0, 8, False, 256), (1, 8, True, 32), (0, 8, True, 32)]
    best_ctas = {0: 4, 2: 16}

    def op_cost(k, cfg):
        fam, c, tc = cfg
        if k == 1:
            return 5.0 if (fam == 1 and tc == 24) else 6.0 if fam == 1 else 9.0
        if fam == 1:
            return 8.0
        return 2.0 if c == best_ctas[k] else 3.0

    class Fake(autograd.CompiledCircuit):
        def __init__(self, penalty):
            self.info = types.SimpleNamespace(n_ops=3)
            self._bshape = [2, 2]
            self.dtype = torch.complex64
            self.device = torch.device("cpu")
            self._plan = None
            self.cfg = [(f, c, tc) for f, c, _, tc in start]
            self.penalty = penalty

        def _params(self, params):
            return params

        def op_config(self, k):
            f, c, tc = self.cfg[k]
            return f, c, start[k][2], tc if tc else start[k][3]

        def tune_op(self, k, family=-1, ctas_per_sm=0, tile_columns=0):
            f, c, tc = self.cfg[k]
            self.cfg[k] = (family if family >= 0 else f, ctas_per_sm or c, tile_columns or tc)

        def _timed_sweeps(self, p, lam, repeats, per_op):
            costs = [op_cost(k, self.cfg[k]) for k in range(3)]
            if per_op:
                return costs, [0.0] * 3
            # the whole step: PDL penalises CTA densities other than 8 by `penalty` each
            return sum(costs) + self.penalty * sum(1 for f, c, _ in self.cfg if f == 0 and c != 8)

    import torch

    c = Fake(penalty=0.0)
    cfgs, before, after = c.autotune(None, ctas=(4, 8, 16), tiles=(32, 24))
    assert cfgs == [(0, 4, 256), (1, 8, 24), (0, 16, 32)] and after < before
    c = Fake(penalty=5.0)  # the CTA picks lose on the whole step: keep densities, take the tile
    cfgs, before, after = c.autotune(None, ctas=(4, 8, 16), tiles=(32, 24))
    assert cfgs == [(0, 8, 256), (1, 8, 24), (0, 8, 32)] and after < before


def _plan_ops(lib, N, D, gates, npar, batch=1, dtype=0):
    from strawberryfields_gb300 import _lib as L

    arr = (L.FockGate * len(gates))()
    for i, g in enumerate(gates):
        arr[i].kind, arr[i].mode1, arr[i].mode2, arr[i].pidx = g
    plan = ctypes.c_void_p()
    L.check(lib.fock_plan_create_batch(N, D, 1, dtype, arr, len(gates), npar, batch, ctypes.byref(plan)))
    info = L.PlanInfo()
    L.check(lib.fock_plan_get_info(plan, ctypes.byref(info)))
    ops = []
    for k in range(info.n_ops):
        a, b, c, d = (ctypes.c_int() for _ in range(4))
        L.check(lib.fock_plan_op(plan, k, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d)))
        g, f, n = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        L.check(lib.fock_plan_op_group(plan, k, ctypes.byref(g), ctypes.byref(f), ctypes.byref(n)))
        ops.append((a.value, b.value, c.value, d.value, g.value, f.value, n.value))
    lib.fock_plan_destroy(plan)
    return ops


@pytest.mark.parametrize("N,D,layers,batch", [(6, 12, 4, 1), (6, 8, 3, 4), (7, 6, 2, 1), (5, 12, 2, 16)])
def test_tile_groups_keep_every_modes_order(lib, monkeypatch, N, D, layers, batch):
    """Fused tile groups (fock_plan_op_group): every op in exactly one group
    or on its own, each group's ops consecutive and within three modes, and
    the ops touching any one mode in the same order as without groups (ops
    are only reordered where they commute)."""
    from strawberryfields_gb300.qnn import qnn_gates

    gates, npar = qnn_gates(N, layers)
    plain = _plan_ops(lib, N, D, gates, npar, batch)  # groups are off by default
    assert all(o[4] == -1 for o in plain)
    monkeypatch.setenv("FOCK_GB300_TILE_GROUPS", "1")
    grouped = _plan_ops(lib, N, D, gates, npar, batch)
    assert len(grouped) == len(plain)
    assert any(o[4] >= 0 for o in grouped)
    for m in range(N):
        seq_p = [o[:4] for o in plain if m in (o[1], o[2])]
        seq_g = [o[:4] for o in grouped if m in (o[1], o[2])]
        assert seq_p == seq_g, m
    k = 0
    while k < len(grouped):
        g, first, count = grouped[k][4:]
        assert first == k
        if g < 0:
            assert count == 1
        else:
            modes = set()
            for j in range(k, k + count):
                assert grouped[j][4] == g
                modes |= {grouped[j][1]} | ({grouped[j][2]} if grouped[j][2] >= 0 else set())
            assert len(modes) <= 3
            assert count >= 2
        k += count


def test_tile_groups_only_where_they_apply(lib, monkeypatch):
    """No groups for complex128, density matrices, cutoffs above 16 or too few
    columns (4 modes at cutoff 15: 15 columns)."""
    from strawberryfields_gb300.qnn import qnn_gates

    monkeypatch.setenv("FOCK_GB300_TILE_GROUPS", "1")
    g6, n6 = qnn_gates(6, 1)
    assert all(o[4] == -1 for o in _plan_ops(lib, 6, 12, g6, n6, dtype=1))
    assert all(o[4] == -1 for o in _plan_ops(lib, 6, 17, g6, n6))
    g4, n4 = qnn_gates(4, 2)
    assert all(o[4] == -1 for o in _plan_ops(lib, 4, 15, g4, n4))
