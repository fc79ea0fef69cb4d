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
    """Per-launch DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum)
    of a kernel class from the committed ncu summaries: lines
    'traffic_bytes_per_launch <class> = <bytes>'."""
    import glob
    import re

    out = {}
    for fn in glob.glob(os.path.join(ROOT, "profiles", "*.md")):
        with open(fn) as f:
            for m in re.finditer(r"^traffic_bytes_per_launch (\S+) = (\d+)", f.read(), re.M):
                out[m.group(1)] = int(m.group(2))
    return out


def _autotune(circ, p):
    cfgs, ms0, ms1 = circ.autotune(p)
    ctas, tiles = {}, {}
    for fam, c, tc in cfgs:
        if fam == 0:
            ctas[str(c)] = ctas.get(str(c), 0) + 1
        else:
            tiles[str(tc)] = tiles.get(str(tc), 0) + 1
    return {"sweep_ms_before": round(ms0, 4), "sweep_ms_after": round(ms1, 4),
            "plane_ops_by_tile_columns": tiles, "block_ops_by_adjoint_ctas_per_sm": ctas}


def gpu_arm(args, rank, world, cpu_base):
    import ctypes

    import torch

    from strawberryfields_gb300 import CompiledCircuit, _lib
    from strawberryfields_gb300.qnn import qnn_params as qnn_params_fn
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
    # per-op kernel family and adjoint CTA density picked by timing (before
    # any capture: tuning reallocates the workspace)
    tune = _autotune(circ, p_dev) if not args.no_autotune else None
    lib = _lib.load()
    # forward + loss + adjoint captured as one CUDA graph (no per-op events
    # inside the timed graph)
    from strawberryfields_gb300.autograd import GraphedGradient

    def loss_fn(psi):
        s = torch.sum(t.conj() * psi)
        return 1 - (s.real ** 2 + s.imag ** 2)

    def run(graphed):
        if graphed is not None:
            loss, g = graphed(p_dev)
        else:
            g, loss = step(p_dev)
        return g

    graphed = None
    if not args.eager:
        graphed = GraphedGradient(circ, loss_fn, p_dev, warmup=1)
        for _ in range(args.warmup):
            graphed(p_dev)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(dev.index)
    clocks.start()
    st = torch.cuda.current_stream(dev)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        evs[k][0].record(st)
        run(graphed)
        evs[k][1].record(st)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    from strawberryfields_gb300.replicas import job_throughput

    value, my_ms = job_throughput(float(np.sum(step_ms)), args.steps)
    ms_per_step = my_ms / args.steps

    # per-op kernel times: the same step with an event before and after every
    # op (a separate capture, after the timed region)
    _lib.check(lib.fock_plan_enable_timing(circ._plan, 1))
    timed = GraphedGradient(circ, loss_fn, p_dev, warmup=1) if not args.eager else None
    nops = circ.n_ops
    fwd_ms = np.zeros(nops, dtype=np.float32)
    bwd_ms = np.zeros(nops, dtype=np.float32)
    fbuf = (ctypes.c_float * nops)()
    bbuf = (ctypes.c_float * nops)()
    op_steps = max(1, min(args.steps, 5))
    for k in range(op_steps):
        flush.zero_()
        run(timed)
        torch.cuda.synchronize()
        _lib.check(lib.fock_plan_op_times(circ._plan, fbuf, bbuf))
        fwd_ms += np.frombuffer(fbuf, dtype=np.float32)
        bwd_ms += np.frombuffer(bbuf, dtype=np.float32)
    _lib.check(lib.fock_plan_enable_timing(circ._plan, 0))
    del timed

    # per-op kernel roofline (averages over the op-timing steps)
    fwd_ms /= op_steps
    bwd_ms /= op_steps
    ops = circ.ops()
    S = circ.info.state_bytes
    peak, peak_kind = _peaks()
    groups = {}
    for k, (kind, m1, m2, nf) in enumerate(ops):
        if circ.op_config(k)[0] == 1:
            name = "plane1" if kind == 1 else "plane2"
        else:
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

    # throughput with a batch of parameter sets: B circuits of the same
    # structure per plan (grid.z), one CUDA graph per step
    batched = None
    if not args.eager and args.batch > 1:
        B = args.batch
        circ_b = CompiledCircuit(N_MODES, CUTOFF, gates, npar, dtype=torch.complex64, device=dev, batch=B)
        pb = torch.stack([torch.tensor(qnn_params_fn(gates, npar, seed=100 + i), device=dev) for i in range(B)])
        tune_b = _autotune(circ_b, pb) if not args.no_autotune else None

        def loss_b(psi):
            s = torch.sum(t.conj() * psi, dim=tuple(range(1, psi.dim())))
            return torch.sum(1 - (s.real ** 2 + s.imag ** 2))

        gb = GraphedGradient(circ_b, loss_b, pb, warmup=1)
        for _ in range(args.warmup):
            gb(pb)
        torch.cuda.synchronize()
        eb0, eb1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        bt = []
        for _ in range(args.steps):
            flush.zero_()
            eb0.record(st)
            gb(pb)
            eb1.record(st)
            eb1.synchronize()
            bt.append(eb0.elapsed_time(eb1))
        ms_b = float(np.median(bt))
        batched = {"circuits_per_step": B, "ms_per_step": ms_b, "grads_per_s": B * 1e3 / ms_b,
                   "autotune": tune_b,
                   "note": "B parameter sets of the same circuit in one batched plan (grid.z), gradient of the "
                           "summed loss w.r.t. every set's parameters"}
        del gb, circ_b

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

    def fwd_ms(c, pp, reps=10):
        for _ in range(3):
            c.forward_states(pp, store_all=False)
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(reps):
            c.forward_states(pp, store_all=False)
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    # the forward configurations: the QNN forward in complex128 too, and the
    # 3-mode cutoff-10 complex128 plain circuit (per mode S and D, BS on
    # (0,1) and (1,2), R and K per mode; seeded parameters)
    c128 = CompiledCircuit(N_MODES, CUTOFF, gates, npar, dtype=torch.complex128, device=dev)
    q128_ms = fwd_ms(c128, p_dev)
    del c128
    g3, np3 = [], 0
    for m in range(3):
        g3 += [(_lib.SQUEEZE, m, -1, np3), (_lib.DISPLACEMENT, m, -1, np3 + 2)]
        np3 += 4
    g3 += [(_lib.BEAMSPLITTER, 0, 1, np3), (_lib.BEAMSPLITTER, 1, 2, np3 + 2)]
    np3 += 4
    for m in range(3):
        g3 += [(_lib.ROTATION, m, -1, np3), (_lib.KERR, m, -1, np3 + 1)]
        np3 += 2
    rng3 = np.random.default_rng(0)
    p3 = torch.tensor(rng3.uniform(0, 0.5, np3), device=dev)
    c3 = CompiledCircuit(3, 10, g3, np3, dtype=torch.complex128, device=dev)
    plain3_ms = fwd_ms(c3, p3, 50)
    del c3
    S64 = circ.info.state_bytes
    flops = circ.info.flops_fwd  # real flops of one forward (the apply kernels' MACs)
    forward_configs = {
        "qnn6x12_complex64": {"ms": 1e3 * fwd_s, "gates_per_s": len(gates) / fwd_s,
                              "gbs": 2 * S64 * nops / fwd_s / 1e9, "fp32_tflops": flops / fwd_s / 1e12},
        "qnn6x12_complex128": {"ms": q128_ms, "gates_per_s": len(gates) / (q128_ms / 1e3),
                               "gbs": 4 * S64 * nops / (q128_ms / 1e3) / 1e9,
                               "fp64_tflops": flops / (q128_ms / 1e3) / 1e12,
                               "fp64_note": "GB300 FP64 is about 1.25 TFLOP/s nominal: the complex128 sweep is "
                                            "FP64-pipe-bound"},
        "plain3x10_complex128": {"us": 1e3 * plain3_ms, "gates_per_s": len(g3) / (plain3_ms / 1e3),
                                 "circuits_per_s": 1e3 / plain3_ms},
        "note": "forward sweeps only (matrix build included), states L2-resident, no flush between reps",
    }

    # end to end through the public API with host buffers: params H2D,
    # gradient + loss D2H every step
    p_host = torch.tensor(params).pin_memory()
    g_host = torch.empty(npar, dtype=torch.float64).pin_memory()
    l_host = torch.empty(1, dtype=torch.float32).pin_memory()
    def e2e_step():
        pd = p_host.to(dev, non_blocking=True)
        if graphed is not None:
            loss, g = graphed(pd)
        else:
            g, loss = step(pd)
        g_host.copy_(g, non_blocking=True)
        l_host.copy_(loss.detach().reshape(1), non_blocking=True)

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(args.steps):
        e2e_step()
    e1.record(st)
    e1.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e2e = {"value": world * 1e3 / e2e_ms, "unit": "grads/s", "h2d_bytes_per_step": npar * 8,
           "d2h_bytes_per_step": npar * 8 + 4, "ms_per_step": e2e_ms}

    # ours per step (as the ncu launch list shows): one matrix build (the
    # adjoint sweep reuses the forward sweep's matrices), nops applies, nops
    # adjoints, one reduction of every op's partial sums, parameter gradients
    launches = 2 * nops + 3
    out = {
        "metric": "CV-QNN grads/s (batched adjoint vs plain kernel+FD, <=1e-5 err); HBM % of peak",
        "value": round(value, 3), "unit": "grads/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 state / fp64 recurrences",
        "data": "synthetic seeded CV-QNN parameters and target",
        "config": _config({"fused_ops": nops, "wall_s_timed": round(wall, 3),
                           "execution": "eager" if graphed is None else "one CUDA graph per step",
                           "autotune": tune}),
        "e2e": e2e, "gpu_launches": launches, "roofline": roof, "kernels": kern,
        "grad_rel_err_vs_fp64": grad_err,
        "fd_baseline": {"gpu_forward_ms": 1e3 * fwd_s, "grads_per_s": fd_grads_per_s,
                        "adjoint_speedup": value / world / fd_grads_per_s},
        "batched_throughput": batched,
        "forward_configs": forward_configs,
        "clocks": clk, "cpu_baseline": cpu_base,
    }
    return out


def single_gate_case(args):
    """Single-gate kernels on a 7-mode cutoff-12 complex64 ket (287 MB, larger
    than L2; --modes / --cutoff choose another): forward apply and adjoint of a squeezer on an inner axis and on
    the last axis, and of a beamsplitter on an inner and on the last adjacent
    pair.  Each op is its own compiled one-gate circuit, timed with the plan's
    per-op events (apply = the apply launch; adjoint = the adjoint launch and
    its partial-sum reduction; the matrix build is outside both).  Bytes per
    launch are 2 S (apply) and 3 S (adjoint); L2 is flushed before each."""
    import ctypes

    import torch

    from strawberryfields_gb300 import CompiledCircuit
    from strawberryfields_gb300 import _lib

    dev = torch.device("cuda", 0)
    lib = _lib.load()
    N, D = args.modes, args.cutoff
    cases = {"dense1_inner": [(4, 2, -1, 0)], "dense1_last": [(4, N - 1, -1, 0)],
             "block2_inner": [(5, 2, 3, 0)], "block2_last": [(5, N - 2, N - 1, 0)]}
    if args.only:
        cases = {k: v for k, v in cases.items() if k in args.only.split(",")}
    rng = np.random.default_rng(0)
    x = torch.as_tensor(rng.normal(size=(D,) * N).astype(np.float32)
                        + 1j * rng.normal(size=(D,) * N).astype(np.float32), device=dev)
    x = (x / torch.linalg.vector_norm(x)).to(torch.complex64)
    lam = x.clone()
    peak, peak_kind = _peaks()
    S = x.numel() * 8
    res = {}
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    fbuf, bbuf = (ctypes.c_float * 1)(), (ctypes.c_float * 1)()
    for name, gates in cases.items():
        circ = CompiledCircuit(N, D, gates, 2, dtype=torch.complex64, device=dev)
        _lib.check(lib.fock_plan_enable_timing(circ._plan, 1))
        p = torch.tensor([0.3, 0.7], device=dev, dtype=torch.float64)
        for _ in range(args.warmup):
            states = circ.forward_states(p, state_in=x)
            circ.backward(p, states, lam, state_in=x)
        ta, tb = [], []
        for _ in range(args.steps):
            flush.zero_()
            states = circ.forward_states(p, state_in=x)
            flush.zero_()
            circ.backward(p, states, lam, state_in=x)
            torch.cuda.synchronize(dev)
            _lib.check(lib.fock_plan_op_times(circ._plan, fbuf, bbuf))
            ta.append(fbuf[0])
            tb.append(bbuf[0])
        ta_ms, tb_ms = float(np.median(ta)), float(np.median(tb))
        res[name] = {"apply_us": 1e3 * ta_ms, "apply_gbs": 2 * S / (ta_ms / 1e3) / 1e9,
                     "adjoint_us": 1e3 * tb_ms, "adjoint_gbs": 3 * S / (tb_ms / 1e3) / 1e9}
        for k in ("apply_gbs", "adjoint_gbs"):
            res[name][k.replace("gbs", "frac")] = res[name][k] / peak
        del circ, states
    print(json.dumps({"case": "single-gate", "state": f"{D}^{N} complex64 ({S / 1e6:.0f} MB)",
                      "note": "kernel time from per-op events: apply = 1 apply launch; adjoint = 1 adjoint "
                              "launch + its partial-sum reduction (median over steps, L2 flushed before each)",
                      "kernels_env": os.environ.get("FOCK_GB300_KERNELS", "default"),
                      "peak_gbs": peak, "peak_source": peak_kind, "kernels": res}))
    return 0


def lossy_case(args):
    """Mixed-state lossy gradient: 4-mode cutoff-14 density matrix (14^8
    complex64 entries, 11.8 GB), 6 CV-QNN layers with a loss channel on every
    mode per layer; loss = mean photon number of mode 0; forward checkpoints
    every 2 layers, each 2-layer segment recomputed recursively in the device
    memory left (a pool of `slots` states).  A step is one forward + one
    adjoint gradient of all parameters.  Checked by the trace of rho and a
    central-difference directional derivative (complex64 forward, h = 1e-2)."""
    import torch

    from strawberryfields_gb300 import CompiledCircuit
    from strawberryfields_gb300.qnn import lossy_qnn_gates, qnn_params

    dev = torch.device("cuda", 0)
    N, D, layers = 4, 14, 6
    gates, npar = lossy_qnn_gates(N, layers)
    params = torch.tensor(qnn_params(gates, npar, seed=0), device=dev)
    # ops per 2 layers (independent of the cutoff)
    n_ops = CompiledCircuit(N, 2, gates, npar, dtype=torch.complex64, device=dev, pure=False).n_ops
    k = 2 * n_ops // layers
    S = 8 * D ** (2 * N)
    free, _ = torch.cuda.mem_get_info(dev)
    n_ckpt = -(-n_ops // k) + 2
    # states: checkpoints + scratch, vacuum input, adjoint pair, pool
    slots = int(min(k - 1, (free - (6 << 30)) // S - n_ckpt - 3))
    if slots < 3:
        print(json.dumps({"case": "lossy", "unavailable": f"{free / 1e9:.0f} GB free: fewer than 3 recompute slots"}))
        return 0
    circ = CompiledCircuit(N, D, gates, npar, dtype=torch.complex64, device=dev, pure=False, checkpoint=k,
                           recompute_slots=slots)
    nvec = torch.arange(D, device=dev, dtype=torch.float32)

    def diag(rho):
        d = rho
        for _ in range(N):
            d = torch.diagonal(d, dim1=0, dim2=1)
        return d  # [D]*N, views only

    def step():
        states = circ.forward_states(params)
        rho = states[circ.final_index()]
        loss = torch.sum(nvec.reshape(D, 1, 1, 1) * diag(rho).real)
        trace = torch.sum(diag(rho).real)
        g = torch.zeros_like(rho)
        diag(g).copy_(nvec.reshape(D, 1, 1, 1).expand(D, D, D, D).to(g.dtype))
        del rho
        grads, _ = circ.backward(params, states, g, overwrite_grad=True)
        del states, g
        return loss, trace, grads

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = []
    for _ in range(args.steps):
        e0.record()
        loss, trace, grads = step()
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    t = float(np.median(times))
    # directional derivative against central differences of the forward
    v = torch.tensor(np.random.default_rng(1).normal(size=npar), device=dev)
    v /= torch.linalg.vector_norm(v)
    h = 1e-2

    def fwd_loss(pp):
        st = circ.forward_states(pp, store_all=False)
        return float(torch.sum(nvec.reshape(D, 1, 1, 1) * diag(st).real))

    fd = (fwd_loss(params + h * v) - fwd_loss(params - h * v)) / (2 * h)
    ad = float(torch.dot(grads, v))
    fwd_ops = n_ops
    print(json.dumps({
        "case": "lossy", "metric": "mixed-state lossy gradients/s", "value": 1.0 / t, "unit": "grads/s",
        "s_per_gradient": t, "steps": args.steps, "warmup": args.warmup,
        "config": {"workload": "4-mode cutoff-14 lossy CV-QNN gradient", "modes": N, "cutoff": D,
                   "layers": layers, "state": f"density matrix 14^8 complex64 ({S / 1e9:.1f} GB)",
                   "gates": len(gates), "params": npar, "ops": n_ops, "checkpoint_every_ops": k,
                   "recompute_slots": slots, "loss": "<n_0>"},
        "loss": float(loss), "trace": float(trace),
        "directional_derivative": {"adjoint": ad, "central_difference": fd,
                                   "rel_err": abs(ad - fd) / max(abs(fd), 1e-30)},
        "state_bytes": S, "forward_op_bytes": 2 * S * fwd_ops,
    }))
    return 0


def batched_case(args):
    """4096 independent CV-QNN circuits, modes U{2..5}, cutoff U{6..20}, depth
    U{2..10} layers (seed 0), complex64: loss and full gradient of every
    circuit per step.  Circuits are grouped by structure into batched compiled
    circuits spread over CUDA streams; groups whose stored states would exceed
    8 GB keep checkpoints."""
    import torch

    from strawberryfields_gb300.batch import CircuitBatch, random_qnn_batch
    from strawberryfields_gb300.qnn import target_state

    dev = torch.device("cuda", 0)
    n = args.circuits
    t0 = time.perf_counter()
    circuits, params = random_qnn_batch(n, seed=0)
    cb = CircuitBatch(circuits, dtype=torch.complex64, device=dev, streams=args.streams)
    setup_s = time.perf_counter() - t0
    targets = {}
    for nm, D, _, _ in circuits:
        if (nm, D) not in targets:
            targets[(nm, D)] = torch.as_tensor(target_state(nm, D, 6, seed=nm * 100 + D), device=dev)
    pt = [torch.tensor(p, device=dev) for p in params]
    flat = torch.cat(pt)
    graphed = None
    if not args.eager:
        t1 = time.perf_counter()
        graphed = cb.capture(pt, targets)
        setup_s += time.perf_counter() - t1
    for _ in range(args.warmup):
        graphed(flat) if graphed else cb.value_and_grad(pt, targets)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(args.steps):
        if graphed:
            losses, grads = graphed(flat)
        else:
            losses, grads = cb.value_and_grad(pt, targets)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    # the graphed step against the eager one (same kernels)
    check = None
    if graphed:
        l_e, g_e = cb.value_and_grad(pt, targets)
        ge = torch.cat([g.reshape(-1) for g in g_e])
        check = {"max_abs_grad_diff_vs_eager": float(torch.max(torch.abs(ge - grads))),
                 "max_abs_loss_diff_vs_eager": float(max(abs(float(a) - float(b)) for a, b in zip(l_e, losses)))}
    stats = cb.stats()
    npar = int(sum(c[3] for c in circuits))
    out = {"case": "batched", "metric": "circuits/s (forward + adjoint gradient of every circuit)",
           "value": n / (ms / 1e3), "unit": "circuits/s", "ms_per_step": ms, "steps": args.steps,
           "warmup": args.warmup, "grads_per_s": n / (ms / 1e3), "params_per_step": npar,
           "config": {"workload": "4096 heterogeneous CV-QNN circuits", "circuits": n, "modes": "U{2..5}",
                      "cutoff": "U{6..20}", "depth": "U{2..10} layers", "seed": 0, "dtype": "complex64"},
           "groups": stats["groups"], "fused_ops": stats["ops"],
           "algorithmic_tb_per_step": (stats["bytes_forward"] + stats["bytes_adjoint"]) / 1e12,
           "achieved_gbs": (stats["bytes_forward"] + stats["bytes_adjoint"]) / (ms / 1e3) / 1e9,
           "setup_s": setup_s, "execution": "eager" if graphed is None else "one CUDA graph per step",
           "graph_check": check}
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--case", default="gradient", choices=["gradient", "single-gate", "batched", "lossy"])
    ap.add_argument("--circuits", type=int, default=4096)
    ap.add_argument("--streams", type=int, default=8, help="batched case: CUDA streams the groups are spread over")
    ap.add_argument("--only", default="", help="single-gate case: comma-separated subset of the kernels")
    ap.add_argument("--modes", type=int, default=7, help="single-gate case: modes of the ket")
    ap.add_argument("--cutoff", type=int, default=12, help="single-gate case: cutoff of the ket")
    ap.add_argument("--eager", action="store_true", help="no CUDA graph capture")
    ap.add_argument("--no-autotune", action="store_true", help="default kernel selection (no per-op tuning)")
    ap.add_argument("--batch", type=int, default=16,
                    help="gradient case: parameter sets per step of the extra batched-throughput line")
    args = ap.parse_args()
    if args.case == "single-gate":
        return single_gate_case(args)
    if args.case == "batched":
        return batched_case(args)
    if args.case == "lossy":
        return lossy_case(args)
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
