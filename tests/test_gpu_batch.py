"""Heterogeneous circuit batches (rows Q1/Q2): circuits of different modes,
cutoffs and depths grouped by structure, each group a batched compiled
circuit; every circuit's loss and gradient against the oracle."""
import numpy as np
import pytest

from oracle import fock_oracle as fo

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_heterogeneous_batch_matches_oracle(cuda, dtype):
    import torch
    from strawberryfields_gb300.batch import CircuitBatch, random_qnn_batch
    from strawberryfields_gb300.qnn import target_state

    circuits, params = random_qnn_batch(14, seed=3, modes=(2, 3), cutoffs=(4, 6), depths=(1, 2))
    tdt = torch.complex128 if dtype == "complex128" else torch.complex64
    # a tiny checkpoint threshold forces the checkpointed sweep on some groups
    cb = CircuitBatch(circuits, dtype=tdt, streams=3, checkpoint_bytes=20_000)
    assert cb.stats()["groups"] < len(circuits) or len(circuits) <= 1
    targets = {}
    for nm, D, _, _ in circuits:
        targets[(nm, D)] = torch.as_tensor(target_state(nm, D, 2, seed=nm * 100 + D), device="cuda")
    pt = [torch.tensor(p, device="cuda") for p in params]
    losses, grads = cb.value_and_grad(pt, targets)
    torch.cuda.synchronize()
    for i, (nm, D, gates, npar) in enumerate(circuits):
        t = targets[(nm, D)].cpu().numpy()
        psi = fo.run_gates(gates, params[i], nm, D)[-1]
        s = np.vdot(t, psi)
        assert abs(losses[i].item() - (1 - abs(s) ** 2)) < (1e-12 if dtype == "complex128" else 1e-5)
        ref = fo.adjoint_grads(gates, params[i], nm, D, -2 * s * t)
        rel = np.linalg.norm(grads[i].cpu().numpy() - ref) / max(np.linalg.norm(ref), 1e-30)
        assert rel < (1e-10 if dtype == "complex128" else 1e-5), (i, rel)


def test_captured_batch_step_matches_eager(cuda):
    """The whole heterogeneous step captured as one CUDA graph (every group's
    forward, loss and adjoint on the group streams) reproduces the eager step
    and follows new parameters copied into its input buffer."""
    import torch
    from strawberryfields_gb300.batch import CircuitBatch, random_qnn_batch
    from strawberryfields_gb300.qnn import target_state

    circuits, params = random_qnn_batch(12, seed=4, modes=(2, 3), cutoffs=(4, 6), depths=(1, 2))
    cb = CircuitBatch(circuits, dtype=torch.complex128, streams=3, checkpoint_bytes=20_000)
    targets = {(nm, D): torch.as_tensor(target_state(nm, D, 2, seed=nm * 100 + D), device="cuda")
               for nm, D, _, _ in circuits}
    pt = [torch.tensor(p, device="cuda") for p in params]
    step = cb.capture(pt, targets)
    for scale in (1.0, 0.7):
        pts = [p * scale for p in pt]
        losses, grads = step(torch.cat(pts))
        l_e, g_e = cb.value_and_grad(pts, targets)
        torch.cuda.synchronize()
        assert torch.allclose(losses, torch.stack([x.reshape(()) for x in l_e]).to(losses.dtype), atol=1e-12)
        ge = torch.cat([g.reshape(-1) for g in g_e])
        assert torch.allclose(grads, ge, atol=1e-12, rtol=1e-12)
        for i in range(len(circuits)):
            o0, o1 = cb.param_offsets[i], cb.param_offsets[i + 1]
            assert torch.allclose(grads[o0:o1], g_e[i].reshape(-1), atol=1e-12)


def test_config4_sample_matches_oracle_in_captured_step(cuda):
    """The 4096-circuit workload's own circuits (modes U{2..5}, cutoff
    U{6..20}, depth U{2..10}, seed 0) in complex64 through the benchmarked
    path -- structure groups on several streams, checkpointed groups, the
    whole step captured as one CUDA graph -- against the oracle: two sampled
    5-mode circuits at cutoff 17-20 and circuits covering every cutoff bucket
    of the kernels (<= 8, 12, 16, 20), mixed with a group of two circuits of
    one structure."""
    import torch
    from strawberryfields_gb300.batch import CircuitBatch, random_qnn_batch
    from strawberryfields_gb300.qnn import target_state

    allc, allp = random_qnn_batch(4096, seed=0)
    pick, seen = [], set()
    # two 5-mode circuits at cutoff >= 17 (the shallow ones: the oracle's
    # cost grows with depth), then one circuit per (cutoff bucket, modes)
    for i, (nm, D, gates, _) in enumerate(allc):
        if nm == 5 and D >= 17 and len(gates) <= 3 * 43 and len([j for j in pick if allc[j][0] == 5]) < 2:
            pick.append(i)
    for i, (nm, D, gates, _) in enumerate(allc):
        bucket = min(b for b in (8, 12, 16, 20) if D <= b)
        if nm < 5 and (bucket, nm) not in seen and len(gates) <= 250:
            seen.add((bucket, nm))
            pick.append(i)
    circuits = [allc[i] for i in pick]
    params = [allp[i] for i in pick]
    # a second circuit with the first 5-mode circuit's structure: a group of two
    circuits.append(circuits[0])
    params.append(np.asarray(params[0]) * 0.9)
    assert any(nm == 5 and D >= 17 for nm, D, _, _ in circuits)
    assert {min(b for b in (8, 12, 16, 20) if D <= b) for _, D, _, _ in circuits} == {8, 12, 16, 20}

    cb = CircuitBatch(circuits, dtype=torch.complex64, streams=4, checkpoint_bytes=64 << 20)
    assert any(g["circ"].checkpoint > 1 for g in cb.groups)
    assert any(len(g["idx"]) > 1 for g in cb.groups)
    targets = {}
    for nm, D, _, _ in circuits:
        if (nm, D) not in targets:
            targets[(nm, D)] = torch.as_tensor(target_state(nm, D, 6, seed=nm * 100 + D), device="cuda")
    pt = [torch.tensor(p, device="cuda") for p in params]
    step = cb.capture(pt, targets)
    losses, grads = step(torch.cat(pt))
    torch.cuda.synchronize()
    losses = losses.cpu().numpy()
    grads = grads.cpu().numpy()
    for i, (nm, D, gates, npar) in enumerate(circuits):
        t = targets[(nm, D)].cpu().numpy()
        psi = fo.run_gates(gates, params[i], nm, D)[-1]
        s = np.vdot(t, psi)
        assert abs(losses[i] - (1 - abs(s) ** 2)) < 1e-5, (i, nm, D)
        ref = fo.adjoint_grads(gates, params[i], nm, D, -2 * s * t)
        got = grads[cb.param_offsets[i]:cb.param_offsets[i + 1]]
        rel = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)
        assert rel < 1e-5, (i, nm, D, len(gates), rel)
