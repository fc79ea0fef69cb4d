"""Generate the phase-space readout golden vectors in this directory from the
reference itself.

Loads the reference package (``oracle/sfref.py``: absent third-party modules
stubbed) and wraps the final states of three committed gate-list fixtures in
the reference's own ``BaseFockState`` (strawberryfields/backends/states.py),
then records

* ``wigner`` (states.py:730) of the first and last mode on a 41 x 37 grid;
* ``x_quad_values`` / ``p_quad_values`` (states.py:436-475) of mode 0;
* ``poly_quad_expectation`` (states.py:806) for seeded quadratic, linear and
  constant coefficients, with and without a quadrature rotation;
* ``quad_expectation`` (states.py:787) of every mode at a few rotation angles.

Output: ``readouts/<case>.npz``.
Usage: python tests/golden/make_readouts.py   (needs the reference sources)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import sfref  # noqa: E402

CASES = ["cfg1_seed0", "mixed_seed0", "mixed_seed1"]
XVEC = np.linspace(-4.0, 4.0, 41)
PVEC = np.linspace(-3.5, 3.5, 37)
QUAD_PHIS = (0.0, np.pi / 4, 1.3, np.pi / 2, 2.9)


def poly_cases(N, seed):
    """(A, d, k, phi) coefficient sets for an N-mode state."""
    rng = np.random.default_rng(seed)
    out = []
    A = np.zeros((2 * N, 2 * N))
    A[0, 0] = 1.0
    out.append((A, None, 0.0, 0.0))                       # <x_0^2>
    A = np.zeros((2 * N, 2 * N))
    A[0, N] = A[N, 0] = 0.5                               # symmetrised x_0 p_0
    out.append((A, np.zeros(2 * N), 0.25, 0.4))
    d = np.zeros(2 * N)
    d[N - 1] = 0.7
    d[2 * N - 1] = -1.3
    out.append((None, d, 0.0, -0.7))                      # linear only, last mode
    B = rng.normal(size=(2 * N, 2 * N))
    out.append(((B + B.T) / 2, rng.normal(size=2 * N), 1.5, 0.3))  # everything, every mode
    if N > 1:
        A = np.zeros((2 * N, 2 * N))
        A[0, 2 * N - 1] = A[2 * N - 1, 0] = 1.0           # x_0 p_{N-1}
        out.append((A, None, 0.0, 1.1))
    return out


def main():
    sf = sfref.import_strawberryfields()
    from strawberryfields.backends.states import BaseFockState

    assert sf is not None
    for case in CASES:
        z = np.load(os.path.join(HERE, case + ".npz"))
        N, D = int(z["N"]), int(z["D"])
        pure = bool(z["out_pure"])
        st = BaseFockState(z["state"], N, pure, D)
        hbar = float(st.hbar)
        W = np.stack([st.wigner(m, XVEC, PVEC) for m in (0, N - 1)])
        xq = st.x_quad_values(0, XVEC, PVEC)
        pq = st.p_quad_values(0, XVEC, PVEC)
        pcs = poly_cases(N, 7)
        As = np.stack([np.zeros((2 * N, 2 * N)) if A is None else A for A, _, _, _ in pcs])
        a_none = np.array([A is None for A, _, _, _ in pcs])
        ds = np.stack([np.zeros(2 * N) if d is None else d for _, d, _, _ in pcs])
        d_none = np.array([d is None for _, d, _, _ in pcs])
        ks = np.array([k for _, _, k, _ in pcs])
        phis = np.array([phi for _, _, _, phi in pcs])
        res = np.array([st.poly_quad_expectation(A, d, k, phi=phi) for A, d, k, phi in pcs])
        qp = np.array(QUAD_PHIS)
        quad = np.array([[st.quad_expectation(m, phi=phi) for phi in qp] for m in range(N)])
        os.makedirs(os.path.join(HERE, "readouts"), exist_ok=True)
        np.savez_compressed(os.path.join(HERE, "readouts", f"{case}.npz"), source=case, hbar=hbar, xvec=XVEC,
                            pvec=PVEC, wigner_modes=np.array([0, N - 1]), wigner=W, x_quad=xq, p_quad=pq,
                            poly_A=As, poly_A_none=a_none, poly_d=ds, poly_d_none=d_none, poly_k=ks,
                            poly_phi=phis, poly_mean_var=res, quad_phis=qp, quad_mean_var=quad)
        print(case, W.shape, res.shape)


if __name__ == "__main__":
    main()
