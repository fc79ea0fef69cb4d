"""Generate the golden vectors in this directory from the reference itself.

Runs the reference's own ``strawberryfields/backends/fockbackend/circuit.py``
``Circuit`` (loaded through ``oracle/sfref.py``: numba absent so its jitted
loops run as numpy; the absent ``thewalrus`` gate matrices served by the
oracle's FP64 restatement) on seeded circuits and stores inputs and outputs:

* ``cfg1_seed{0,1,2}``: 3 modes, cutoff 10, complex128: vacuum; per mode
  Sgate(r~U[0,.5], phi~U[0,2pi]) and Dgate(|a|~U[0,.5], arg~U[0,2pi]);
  BSgate(theta~U[0,pi/2], phi~U[0,2pi]) on (0,1) and (1,2); Rgate(U[0,2pi])
  and Kgate(kappa~U[0,.1]) per mode -- the 3-mode cutoff-10 plain circuit.
* ``mixed_seed{0,1}``: 2 modes, cutoff 6, mixed: squeezers, beamsplitters,
  two-mode squeezer, MZ, cross-Kerr and loss channels.
* ``pure_all_seed0``: 3 modes, cutoff 7, every pure gate kind incl. swapped
  and non-adjacent mode pairs with mode2 != 0.
* ``homodyne_{pure,mixed}_seed0``: gates, a homodyne measurement with a
  post-selected value ("MH": phi, value, mode; circuit.py:713-801 without the
  sampling), then more gates.
* ``swapped_mixed_seed0``: the same kinds with mode pairs (2, 0) and (1, 0),
  run on a mixed state.  The reference's pure-state two-mode path
  (fockbackend/circuit.py:242-248) moves the wrong axes to the front when
  mode2 == 0 and disagrees with its own mixed-state path there; the
  mixed-state path follows the gate definitions and is the one pinned.

Usage: python tests/golden/make_golden.py   (needs the reference sources)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import sfref  # noqa: E402

# op codes stored in the fixtures: (name, params..., modes...)
OPS = {"S": 1, "D": 2, "BS": 3, "R": 4, "K": 5, "S2": 6, "MZ": 7, "CK": 8, "L": 9, "MH": 10}


def cfg1(seed):
    rng = np.random.default_rng(seed)
    ops = []
    for m in range(3):
        ops.append(("S", rng.uniform(0, 0.5), rng.uniform(0, 2 * np.pi), m))
        ops.append(("D", rng.uniform(0, 0.5), rng.uniform(0, 2 * np.pi), m))
    for pair in [(0, 1), (1, 2)]:
        ops.append(("BS", rng.uniform(0, np.pi / 2), rng.uniform(0, 2 * np.pi)) + pair)
    for m in range(3):
        ops.append(("R", rng.uniform(0, 2 * np.pi), m))
        ops.append(("K", rng.uniform(0, 0.1), m))
    return 3, 10, True, ops


def mixed(seed):
    rng = np.random.default_rng(100 + seed)
    u = rng.uniform
    ops = [("S", u(0, .4), u(0, 6.28), 0), ("BS", u(0, 1.5), u(0, 6.28), 0, 1), ("L", u(.7, 1), 1),
           ("D", u(0, .4), u(0, 6.28), 1), ("S2", u(0, .3), u(0, 6.28), 1, 0), ("K", u(0, .1), 0),
           ("MZ", u(0, 6.28), u(0, 6.28), 0, 1), ("CK", u(0, .1), 0, 1), ("L", u(.7, 1), 0),
           ("R", u(0, 6.28), 1), ("BS", u(0, 1.5), u(0, 6.28), 1, 0)]
    return 2, 6, False, ops


def pure_all(seed):
    rng = np.random.default_rng(200 + seed)
    u = rng.uniform
    ops = [("S", u(0, .4), u(0, 6.28), 1), ("D", u(0, .4), u(0, 6.28), 2), ("BS", u(0, 1.5), u(0, 6.28), 2, 1),
           ("S2", u(0, .3), u(0, 6.28), 0, 2), ("R", u(0, 6.28), 0), ("MZ", u(0, 6.28), u(0, 6.28), 1, 2),
           ("K", u(0, .1), 1), ("CK", u(0, .1), 2, 0), ("BS", u(0, 1.5), u(0, 6.28), 0, 1),
           ("D", u(0, .4), u(0, 6.28), 0), ("S2", u(0, .3), u(0, 6.28), 2, 1)]
    return 3, 7, True, ops


def swapped_mixed(seed):
    rng = np.random.default_rng(300 + seed)
    u = rng.uniform
    ops = [("S", u(0, .4), u(0, 6.28), 0), ("D", u(0, .4), u(0, 6.28), 2), ("BS", u(0, 1.5), u(0, 6.28), 2, 0),
           ("S2", u(0, .3), u(0, 6.28), 1, 0), ("MZ", u(0, 6.28), u(0, 6.28), 2, 0), ("K", u(0, .1), 1),
           ("BS", u(0, 1.5), u(0, 6.28), 1, 0), ("D", u(0, .4), u(0, 6.28), 1)]
    return 3, 5, False, ops


def homodyne(seed, pure):
    rng = np.random.default_rng(400 + seed + (0 if pure else 50))
    u = rng.uniform
    ops = [("S", u(0, .4), u(0, 6.28), 0), ("D", u(0, .5), u(0, 6.28), 1), ("BS", u(0, 1.5), u(0, 6.28), 0, 1)]
    if not pure:
        ops.append(("L", u(.7, 1), 1))
    ops += [("MH", u(0, 6.28), u(-1.5, 1.5), 0), ("D", u(0, .4), u(0, 6.28), 0), ("BS", u(0, 1.5), u(0, 6.28), 0, 1)]
    return 2, 8 if pure else 6, pure, ops


def run_reference(N, D, pure, ops):
    _, Circuit = sfref.load_fock_circuit()
    c = Circuit(N, D, pure=pure)
    for op in ops:
        name, rest = op[0], op[1:]
        if name == "S":
            c.squeeze(rest[0], rest[1], rest[2])
        elif name == "D":
            c.displacement(rest[0], rest[1], rest[2])
        elif name == "BS":
            c.beamsplitter(rest[0], rest[1], rest[2], rest[3])
        elif name == "R":
            c.phase_shift(rest[0], rest[1])
        elif name == "K":
            c.kerr_interaction(rest[0], rest[1])
        elif name == "S2":
            c.two_mode_squeeze(rest[0], rest[1], rest[2], rest[3])
        elif name == "MZ":
            c.mzgate(rest[0], rest[1], rest[2], rest[3])
        elif name == "CK":
            c.cross_kerr_interaction(rest[0], rest[1], rest[2])
        elif name == "L":
            c.loss(rest[0], rest[1])
        elif name == "MH":
            c.measure_homodyne(rest[0], rest[2], select=rest[1])
    state, is_pure = c.get_state()
    return np.asarray(state, dtype=np.complex128), is_pure


def encode(ops):
    """ops -> float array rows [code, p0, p1, m1, m2] (p1/m2 = nan/-1 if absent)."""
    rows = []
    for op in ops:
        name = op[0]
        if name in ("S", "D", "BS", "S2", "MZ", "MH"):
            p = op[1:3]
            modes = op[3:]
        else:
            p = op[1:2]
            modes = op[2:]
        rows.append([OPS[name], p[0], p[1] if len(p) > 1 else np.nan, modes[0], modes[1] if len(modes) > 1 else -1])
    return np.array(rows, dtype=np.float64)


def decode(arr):
    inv = {v: k for k, v in OPS.items()}
    ops = []
    for code, p0, p1, m1, m2 in arr:
        name = inv[int(code)]
        ps = [p0] if np.isnan(p1) else [p0, p1]
        ms = [int(m1)] if int(m2) < 0 else [int(m1), int(m2)]
        ops.append(tuple([name] + ps + ms))
    return ops


def main():
    cases = {}
    for s in range(3):
        cases[f"cfg1_seed{s}"] = cfg1(s)
    for s in range(2):
        cases[f"mixed_seed{s}"] = mixed(s)
    cases["pure_all_seed0"] = pure_all(0)
    cases["homodyne_pure_seed0"] = homodyne(0, True)
    cases["homodyne_mixed_seed0"] = homodyne(0, False)
    cases["swapped_mixed_seed0"] = swapped_mixed(0)
    for name, (N, D, pure, ops) in cases.items():
        state, is_pure = run_reference(N, D, pure, ops)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), N=N, D=D, pure=pure, ops=encode(ops),
                            state=state, out_pure=is_pure)
        print(name, state.shape, "pure" if is_pure else "mixed")


if __name__ == "__main__":
    main()
