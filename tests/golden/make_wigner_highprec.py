"""High-precision Wigner values for the device kernel's wide-range test.

At large cutoffs and far from the origin the Wigner sum cancels terms many
orders of magnitude larger than the result, and a double-precision
evaluation of either recurrence (the reference's iteration,
strawberryfields/backends/states.py:730-785, or the Laguerre form) loses
digits.  This script evaluates W_{|m><m+k|} from its Laguerre form
(e^{-2|A|^2}/pi (2A)^k (-1)^m sqrt(m!/(m+k)!) L_m^k(4|A|^2), A = (x+ip)/sqrt(2 hbar))
in 50-digit arithmetic (mpmath) for seeded random density matrices and
stores the results.

Output: ``highprec/wigner.npz``.  Usage: python tests/golden/make_wigner_highprec.py
"""
import os

import mpmath
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
mpmath.mp.dps = 50


def rho_of(D, seed):
    rng = np.random.default_rng(seed)
    Z = rng.normal(size=(D, D)) + 1j * rng.normal(size=(D, D))
    rho = Z @ Z.conj().T
    return rho / np.trace(rho)


def wigner_point(rho, x, p, hbar):
    D = rho.shape[0]
    A = (mpmath.mpf(x) + 1j * mpmath.mpf(p)) / mpmath.sqrt(2 * mpmath.mpf(hbar))
    y = 4 * abs(A) ** 2
    W = mpmath.mpf(0)
    for k in range(D):
        # sum_m rho[m][m+k] (-1)^m sqrt(m!/(m+k)!) L_m^k(y) by the exact recurrence
        # L_{m+1} = ((2m+1+k-y) L_m - (m+k) L_{m-1}) / (m+1)
        Lm1, Lm = mpmath.mpf(0), mpmath.mpf(1)
        s = mpmath.mpc(0)
        for m in range(D - k):
            c = (-1) ** m * mpmath.sqrt(mpmath.factorial(m) / mpmath.factorial(m + k))
            r = rho[m, m + k]
            s += mpmath.mpc(r.real, r.imag) * c * Lm
            Lm1, Lm = Lm, ((2 * m + 1 + k - y) * Lm - (m + k) * Lm1) / (m + 1)
        t = (mpmath.exp(-y / 2) / mpmath.pi * (2 * A) ** k * s).real
        W += t if k == 0 else 2 * t
    return W / hbar


def main():
    out = {}
    for D, seed in ((30, 30), (64, 64)):
        rho = rho_of(D, seed)
        xv = np.linspace(-9, 9, 7)
        pv = np.linspace(-7, 8, 6)
        hbar = 1.3
        W = np.array([[float(wigner_point(rho, x, p, hbar)) for x in xv] for p in pv])
        out[f"rho{D}"], out[f"x{D}"], out[f"p{D}"], out[f"w{D}"] = rho, xv, pv, W
        print(D, np.abs(W).max())
    os.makedirs(os.path.join(HERE, "highprec"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "highprec", "wigner.npz"), hbar=1.3, **out)


if __name__ == "__main__":
    main()
