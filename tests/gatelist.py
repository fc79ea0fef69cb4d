"""Golden-fixture op lists (tests/golden/make_golden.py) as compiled-circuit
gate lists: (kind, mode1, mode2, parameter index) plus the parameter vector."""

KINDS = {"R": 1, "K": 2, "D": 3, "S": 4, "BS": 5, "S2": 6, "MZ": 7, "CK": 8, "L": 9}
NPAR = {"R": 1, "K": 1, "D": 2, "S": 2, "BS": 2, "S2": 2, "MZ": 2, "CK": 1, "L": 1}


def ops_to_gates(ops):
    gates, params = [], []
    for op in ops:
        name, rest = op[0], op[1:]
        n = NPAR[name]
        modes = rest[n:]
        gates.append((KINDS[name], int(modes[0]), int(modes[1]) if len(modes) > 1 else -1, len(params)))
        params += [float(v) for v in rest[:n]]
    return gates, params
