#!/usr/bin/env python3
"""Benchmark: CV-QNN gradients per second on one GB300 (and replicas on N).

Workload (one "step" = one full gradient): the 6-mode, cutoff-12, 4-layer
CV-QNN circuit (layer of examples/quantum_neural_network.py; 232 gates, 400
real parameters, ket of 12^6 = 2.99e6 amplitudes), complex64 state with FP64
gate recurrences, loss 1 - |<psi_t|psi>|^2 against a seeded target restricted
to total photon number <= 6.  A step runs the fused forward sweep (168 ops:
rotations and Kerr gates are folded into neighbouring gates), the loss in
torch, and the adjoint sweep that yields all 400 derivatives.

Reported beside it: gradient error of the complex64 result against the
complex128 (FP64) GPU gradient, the plain-GPU-forward + central-differences
baseline of the same circuit ((2P+1) forwards per gradient), per-kernel
roofline figures from CUDA events recorded between the ops of the timed
steps, and the reference's own CPU implementation (its fockbackend Circuit)
timed on a bounded sample of the circuit on all host cores.

--impl reference runs only that CPU measurement (rank 0; other ranks exit).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_MODES, CUTOFF, LAYERS = 6, 12, 4
PARAM_SEED, TARGET_SEED, TARGET_PHOTONS = 0, 1, 6


def _workload():
    from strawberryfields_gb300.qnn import qnn_gates, qnn_params

    gates, npar = qnn_gates(N_MODES, LAYERS)
    params = qnn_params(gates, npar, PARAM_SEED, r_max=0.3, a_max=0.3, k_max=0.05)
    return gates, npar, params


def _config(extra=None):
    cfg = {"workload": "cvqnn-adjoint-gradient", "modes": N_MODES, "cutoff": CUTOFF, "layers": LAYERS,
           "gates": 232, "params": 400, "state": "pure ket 12^6 complex64", "recurrences": "fp64",
           "loss": "1-|<psi_t|psi>|^2, target total photons <= 6", "l2": "flushed between steps (256 MB write)",
           "parallelism": "replicas"}
    if extra:
        cfg.update(extra)
    return cfg


# ---------------------------------------------------------------------------
# reference CPU implementation (bounded sample, all host cores)
# ---------------------------------------------------------------------------
def _ref_worker(args):
    """Time the reference fockbackend Circuit on one sample of each gate kind
    (runs in a spawned process)."""
    sys.path.insert(0, ROOT)
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    from oracle import sfref

    ops_mod, Circuit = sfref.load_fock_circuit()
    rng = np.random.default_rng(args)
    c = Circuit(N_MODES, CUTOFF, pure=True)
    # a non-trivial state first (not timed)
    for m in range(N_MODES):
        c.squeeze(0.1, 0.2, m)
    times = {}
    samples = [("squeeze", lambda: c.squeeze(rng.uniform(0, .3), rng.uniform(0, 6.28), 2)),
               ("displacement", lambda: c.displacement(rng.uniform(0, .3), rng.uniform(0, 6.28), 3)),
               ("beamsplitter", lambda: c.beamsplitter(rng.uniform(0, 1.5), rng.uniform(0, 6.28), 2, 3)),
               ("rotation", lambda: c.phase_shift(rng.uniform(0, 6.28), 1)),
               ("kerr", lambda: c.kerr_interaction(rng.uniform(0, .05), 4))]
    for name, fn in samples:
        t0 = time.perf_counter()
        fn()
        times[name] = time.perf_counter() - t0
    return times


def reference_cpu(steps, warmup):
    """Grads/s of the reference's CPU path: (2P+1)-forward central differences
    with the reference Circuit, the 2P+1 forwards spread over all host cores.
    Each step times one sample of every gate kind in every worker and
    extrapolates to the 232-gate circuit."""
    import multiprocessing as mp

    from strawberryfields_gb300.qnn import qnn_gates

    gates, npar = qnn_gates(N_MODES, LAYERS)
    counts = {"squeeze": 0, "displacement": 0, "beamsplitter": 0, "rotation": 0, "kerr": 0}
    names = {1: "rotation", 2: "kerr", 3: "displacement", 4: "squeeze", 5: "beamsplitter"}
    for g in gates:
        counts[names[g[0]]] += 1
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    vals = []
    sample_s = []
    with ctx.Pool(cores) as pool:
        for it in range(warmup + steps):
            t0 = time.perf_counter()
            res = pool.map(_ref_worker, [1000 * it + w for w in range(cores)])
            wall = time.perf_counter() - t0
            # per-worker forward time estimate; all workers ran concurrently
            fwd = [sum(counts[k] * r[k] for k in counts) for r in res]
            t_fwd = float(np.mean(fwd))
            grads_per_s = cores / ((2 * npar + 1) * t_fwd)
            if it >= warmup:
                vals.append(grads_per_s)
                sample_s.append(wall)
    return {
        "value": float(np.median(vals)),
        "unit": "grads/s",
        "cores": cores,
        "kind": "reference",
        "sample": (f"reference fockbackend Circuit (numba absent: its jitted loops run as numpy; thewalrus "
                   f"matrices from the FP64 restatement), one squeeze/displacement/beamsplitter/rotation/Kerr "
                   f"on the 12^6 complex128 ket per worker, {cores} concurrent workers, extrapolated to 232 "
                   f"gates x (2*{npar}+1) central-difference forwards; {np.mean(sample_s):.1f} s per step"),
        "forward_s_per_worker": t_fwd,
    }


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
class ClockSampler:
    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def _traffic():
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def gpu_arm(args, rank, world, cpu_base):
    import ctypes

    import torch

    from strawberryfields_gb300 import CompiledCircuit, _lib
    from strawberryfields_gb300.qnn import target_state

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    gates, npar, params = _workload()
    circ = CompiledCircuit(N_MODES, CUTOFF, gates, npar, dtype=torch.complex64, device=dev)
    t = torch.as_tensor(target_state(N_MODES, CUTOFF, TARGET_PHOTONS, TARGET_SEED), device=dev).to(torch.complex64)
    p_dev = torch.tensor(params, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step(p):
        p = p.detach().requires_grad_(True)
        psi = circ(p)
        s = torch.sum(t.conj() * psi)
        loss = 1 - (s.real ** 2 + s.imag ** 2)
        loss.backward()
        return p.grad, loss

    for _ in range(args.warmup):
        step(p_dev)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    lib = _lib.load()
    _lib.check(lib.fock_plan_enable_timing(circ._plan, 1))
    nops = circ.n_ops
    fwd_ms = np.zeros(nops, dtype=np.float32)
    bwd_ms = np.zeros(nops, dtype=np.float32)
    fbuf = (ctypes.c_float * nops)()
    bbuf = (ctypes.c_float * nops)()
    clocks = ClockSampler(dev.index)
    clocks.start()
    st = torch.cuda.current_stream(dev)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        evs[k][0].record(st)
        g, loss = step(p_dev)
        evs[k][1].record(st)
        evs[k][1].synchronize()
        _lib.check(lib.fock_plan_op_times(circ._plan, fbuf, bbuf))
        fwd_ms += np.frombuffer(fbuf, dtype=np.float32)
        bwd_ms += np.frombuffer(bbuf, dtype=np.float32)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    _lib.check(lib.fock_plan_enable_timing(circ._plan, 0))
    step_ms = [a.elapsed_time(b) for a, b in evs]
    from strawberryfields_gb300.replicas import job_throughput

    value, my_ms = job_throughput(float(np.sum(step_ms)), args.steps)
    ms_per_step = my_ms / args.steps

    # per-op kernel roofline (averages over the timed steps)
    fwd_ms /= args.steps
    bwd_ms /= args.steps
    ops = circ.ops()
    S = circ.info.state_bytes
    peak, peak_kind = _peaks()
    groups = {}
    for k, (kind, m1, m2, nf) in enumerate(ops):
        name = "dense1" if kind == 1 else "block2"
        for direction, arr, bytes_per in (("apply", fwd_ms, 2 * S), ("adjoint", bwd_ms, 3 * S)):
            key = f"{direction}_{name}"
            gsum = groups.setdefault(key, {"launches": 0, "ms": 0.0, "bytes": 0})
            gsum["launches"] += 1
            gsum["ms"] += float(arr[k])
            gsum["bytes"] += bytes_per
    kern = {}
    for key, gsum in groups.items():
        avg = gsum["ms"] / gsum["launches"]
        kern[key] = {"launches_per_step": gsum["launches"], "avg_launch_us": 1e3 * avg,
                     "share_of_sweeps": gsum["ms"] / float(fwd_ms.sum() + bwd_ms.sum()),
                     "algorithmic_gb_per_launch": gsum["bytes"] / gsum["launches"] / 1e9,
                     "achieved_gbs": gsum["bytes"] / gsum["launches"] / (avg / 1e3) / 1e9}
    dom = max(kern, key=lambda k: kern[k]["share_of_sweeps"])
    traffic = _traffic().get(dom)
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(kern[dom]["achieved_gbs"], 1), "peak": peak,
            "unit": "GB/s", "frac": round(kern[dom]["achieved_gbs"] / peak, 4),
            "traffic": traffic, "peak_source": peak_kind,
            "algorithmic_bytes_per_launch": kern[dom]["algorithmic_gb_per_launch"] * 1e9}

    # gradient error against the FP64 (complex128) GPU gradient
    circ128 = CompiledCircuit(N_MODES, CUTOFF, gates, npar, dtype=torch.complex128, device=dev)
    t128 = t.to(torch.complex128)
    p = p_dev.detach().clone().requires_grad_(True)
    psi = circ128(p)
    s = torch.sum(t128.conj() * psi)
    (1 - torch.abs(s) ** 2).backward()
    g128 = p.grad.detach()
    g64, _ = step(p_dev)
    grad_err = float(torch.linalg.vector_norm(g64 - g128) / torch.linalg.vector_norm(g128))
    del circ128, psi

    # plain GPU forward + central differences
    for _ in range(3):
        circ.forward_states(p_dev, store_all=False)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nrep = 10
    e0.record(st)
    for _ in range(nrep):
        circ.forward_states(p_dev, store_all=False)
    e1.record(st)
    e1.synchronize()
    fwd_s = e0.elapsed_time(e1) / nrep / 1e3
    fd_grads_per_s = 1.0 / ((2 * npar + 1) * fwd_s)

    # end to end through the public API with host buffers: params H2D,
    # gradient + loss D2H every step
    p_host = torch.tensor(params).pin_memory()
    g_host = torch.empty(npar, dtype=torch.float64).pin_memory()
    l_host = torch.empty(1, dtype=torch.float32).pin_memory()
    for _ in range(args.warmup):
        pd = p_host.to(dev, non_blocking=True)
        g, loss = step(pd)
        g_host.copy_(g, non_blocking=True)
        l_host.copy_(loss.detach().reshape(1), non_blocking=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(args.steps):
        pd = p_host.to(dev, non_blocking=True)
        g, loss = step(pd)
        g_host.copy_(g, non_blocking=True)
        l_host.copy_(loss.detach().reshape(1), non_blocking=True)
    e1.record(st)
    e1.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e2e = {"value": world * 1e3 / e2e_ms, "unit": "grads/s", "h2d_bytes_per_step": npar * 8,
           "d2h_bytes_per_step": npar * 8 + 4, "ms_per_step": e2e_ms}

    launches = 2 * nops + 4
    out = {
        "metric": "CV-QNN grads/s (batched adjoint vs plain kernel+FD, <=1e-5 err); HBM % of peak",
        "value": round(value, 3), "unit": "grads/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 state / fp64 recurrences",
        "data": "synthetic seeded CV-QNN parameters and target",
        "config": _config({"fused_ops": nops, "wall_s_timed": round(wall, 3)}),
        "e2e": e2e, "gpu_launches": launches, "roofline": roof, "kernels": kern,
        "grad_rel_err_vs_fp64": grad_err,
        "fd_baseline": {"gpu_forward_ms": 1e3 * fwd_s, "grads_per_s": fd_grads_per_s,
                        "adjoint_speedup": value / world / fd_grads_per_s},
        "clocks": clk, "cpu_baseline": cpu_base,
    }
    return out


def single_gate_case(args):
    """Single-gate kernels on a 7-mode cutoff-12 complex64 ket (287 MB, larger
    than L2): forward apply and adjoint of a squeezer on an inner axis and on
    the last axis, and of a beamsplitter on an inner and on the last adjacent
    pair.  Each op is its own compiled one-gate circuit; bytes per launch are
    2 S (apply) and 3 S (adjoint)."""
    import torch

    from strawberryfields_gb300 import CompiledCircuit

    dev = torch.device("cuda", 0)
    N, D = 7, 12
    cases = {"dense1_inner": [(4, 2, -1, 0)], "dense1_last": [(4, 6, -1, 0)],
             "block2_inner": [(5, 2, 3, 0)], "block2_last": [(5, 5, 6, 0)]}
    rng = np.random.default_rng(0)
    x = torch.as_tensor(rng.normal(size=(D,) * N).astype(np.float32)
                        + 1j * rng.normal(size=(D,) * N).astype(np.float32), device=dev)
    x = (x / torch.linalg.vector_norm(x)).to(torch.complex64)
    lam = x.clone()
    peak, peak_kind = _peaks()
    S = x.numel() * 8
    res = {}
    st = torch.cuda.current_stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for name, gates in cases.items():
        circ = CompiledCircuit(N, D, gates, 2, dtype=torch.complex64, device=dev)
        p = torch.tensor([0.3, 0.7], device=dev, dtype=torch.float64)
        for _ in range(args.warmup):
            states = circ.forward_states(p, state_in=x)
            circ.backward(p, states, lam, state_in=x)
        ta, tb = [], []
        for _ in range(args.steps):
            flush.zero_()
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(st)
            states = circ.forward_states(p, state_in=x)
            e1.record(st)
            flush.zero_()
            e3 = torch.cuda.Event(enable_timing=True)
            e3.record(st)
            circ.backward(p, states, lam, state_in=x)
            e2.record(st)
            e2.synchronize()
            ta.append(e0.elapsed_time(e1))
            tb.append(e3.elapsed_time(e2))
        ta_ms, tb_ms = float(np.median(ta)), float(np.median(tb))
        res[name] = {"apply_us": 1e3 * ta_ms, "apply_gbs": 2 * S / (ta_ms / 1e3) / 1e9,
                     "adjoint_us": 1e3 * tb_ms, "adjoint_gbs": 3 * S / (tb_ms / 1e3) / 1e9}
        for k in ("apply_gbs", "adjoint_gbs"):
            res[name][k.replace("gbs", "frac")] = res[name][k] / peak
        del circ, states
    print(json.dumps({"case": "single-gate", "state": f"{D}^{N} complex64 ({S / 1e6:.0f} MB)",
                      "note": "apply = build + 1 apply launch; adjoint = build + 1 adjoint launch + reduce + "
                              "param-grad launches (event span)",
                      "peak_gbs": peak, "peak_source": peak_kind, "kernels": res}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--case", default="gradient", choices=["gradient", "single-gate"])
    args = ap.parse_args()
    if args.case == "single-gate":
        return single_gate_case(args)
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))

    if args.impl == "reference":
        if rank != 0:
            return 0
        base = reference_cpu(args.steps, args.warmup)
        line = {"impl": "reference",
                "metric": "CV-QNN grads/s (batched adjoint vs plain kernel+FD, <=1e-5 err); HBM % of peak",
                "value": base["value"], "unit": "grads/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "c128 (reference precision)", "data": "synthetic seeded CV-QNN parameters",
                "config": _config({"arm": "reference fockbackend Circuit, central differences"}),
                "cpu_baseline": base,
                "e2e": {"value": base["value"], "unit": "grads/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    # CPU baseline first: its spawn pool starts before any GPU work
    cpu_base = None
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            cpu_base = reference_cpu(1, 0)
        except Exception as e:  # reference sources absent
            cpu_base = {"unavailable": f"{type(e).__name__}: {e}"}
    if world > 1:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        torch.distributed.init_process_group("nccl")
    out = gpu_arm(args, rank, world, cpu_base)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
