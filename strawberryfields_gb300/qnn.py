"""CV quantum neural network circuits as gate lists.

Layer structure of the reference example ``examples/quantum_neural_network.py``
(``interferometer`` :14-50, ``layer`` :55-85): a rectangular mesh of
beamsplitters on adjacent pairs followed by rotations on the first N-1 modes,
squeezers on every mode, a second mesh, then displacement and Kerr on every
mode.  Parameters are drawn from ``numpy.random.default_rng(seed)`` with the
ranges of the synthetic workloads: theta ~ U[0, pi/2] and phases ~ U[0, 2 pi]
for the meshes, |r| ~ U[0, r_max] for squeezing (phase U[0, 2 pi]),
|alpha| ~ U[0, a_max] (arg U[0, 2 pi]) for displacement, kappa ~ U[0, k_max].
"""

import numpy as np

from . import _lib as L


def interferometer_gates(N, pidx, gates):
    """Append the mesh of one interferometer; return the next free param index."""
    if N == 1:
        gates.append((L.ROTATION, 0, -1, pidx))
        return pidx + 1
    for l in range(N):
        for k in range(N - 1):
            if (l + k) % 2 != 1:
                gates.append((L.BEAMSPLITTER, k, k + 1, pidx))
                pidx += 2
    for i in range(max(1, N - 1)):
        gates.append((L.ROTATION, i, -1, pidx))
        pidx += 1
    return pidx


def qnn_gates(N, layers):
    """Gate list and parameter count of an N-mode, ``layers``-deep CV-QNN.

    Every gate owns its parameters: BS (theta, phi), R (phi), S (r, phi),
    D (|alpha|, arg), K (kappa)."""
    gates = []
    p = 0
    for _ in range(layers):
        p = interferometer_gates(N, p, gates)
        for i in range(N):
            gates.append((L.SQUEEZE, i, -1, p))
            p += 2
        p = interferometer_gates(N, p, gates)
        for i in range(N):
            gates.append((L.DISPLACEMENT, i, -1, p))
            p += 2
            gates.append((L.KERR, i, -1, p))
            p += 1
    return gates, p


def lossy_qnn_gates(N, layers):
    """``qnn_gates`` with a loss channel on every mode at the end of every
    layer (the mixed-state lossy workload: LossChannel(T) per mode per layer,
    reference ops.py LossChannel / fockbackend/circuit.py:65-87)."""
    gates, p = [], 0
    for _ in range(layers):
        layer, n = qnn_gates(N, 1)
        gates += [(k, m1, m2, pi + p) for k, m1, m2, pi in layer]
        p += n
        for m in range(N):
            gates.append((L.LOSS, m, -1, p))
            p += 1
    return gates, p


def qnn_params(gates, n_params, seed, r_max=0.3, a_max=0.3, k_max=0.05, t_min=0.8):
    """Seeded parameter vector for a ``qnn_gates`` list."""
    rng = np.random.default_rng(seed)
    p = np.zeros(n_params)
    for kind, _m1, _m2, i in gates:
        if kind == L.BEAMSPLITTER:
            p[i] = rng.uniform(0, np.pi / 2)
            p[i + 1] = rng.uniform(0, 2 * np.pi)
        elif kind == L.ROTATION:
            p[i] = rng.uniform(0, 2 * np.pi)
        elif kind == L.SQUEEZE:
            p[i] = rng.uniform(0, r_max)
            p[i + 1] = rng.uniform(0, 2 * np.pi)
        elif kind == L.DISPLACEMENT:
            p[i] = rng.uniform(0, a_max)
            p[i + 1] = rng.uniform(0, 2 * np.pi)
        elif kind == L.KERR:
            p[i] = rng.uniform(0, k_max)
        elif kind == L.LOSS:
            p[i] = rng.uniform(t_min, 1.0)
    return p


def target_state(N, D, max_photons, seed):
    """Seeded complex Gaussian target, zero outside total photon number
    <= ``max_photons``, normalised (loss 1 - |<target|psi>|^2)."""
    rng = np.random.default_rng(seed)
    t = rng.normal(size=(D,) * N) + 1j * rng.normal(size=(D,) * N)
    tot = np.zeros((D,) * N, dtype=np.int64)
    for m in range(N):
        shape = [1] * N
        shape[m] = D
        tot = tot + np.arange(D).reshape(shape)
    t[tot > max_photons] = 0
    return t / np.linalg.norm(t)
