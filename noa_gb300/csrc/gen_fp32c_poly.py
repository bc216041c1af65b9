"""Coefficients of H(u) = (log1p(u) - u) / u^2 on [0, 1] for dcs_fp32c.cuh.

log1p(u)/u - 1 = u H(u) cancels catastrophically when evaluated directly for
small u; the polynomial does not.  Chebyshev least-squares fit at 200 nodes
(mpmath, 40 digits), converted to monomial form and rounded to float.

    python noa_gb300/csrc/gen_fp32c_poly.py
"""
import mpmath
import numpy as np

mpmath.mp.dps = 40
DEG = 9


def H(u):
    u = mpmath.mpf(u)
    return mpmath.mpf(-0.5) if u == 0 else (mpmath.log1p(u) - u) / u ** 2


def main():
    n = 200
    xs = [0.5 * (1 - mpmath.cos(mpmath.pi * (k + 0.5) / n)) for k in range(n)]
    fit = np.polynomial.chebyshev.Chebyshev.fit([float(x) for x in xs], [float(H(x)) for x in xs], DEG,
                                                domain=[0, 1])
    coef = fit.convert(kind=np.polynomial.Polynomial).coef
    err = max(abs(np.polynomial.polynomial.polyval(float(t), coef) - float(H(t))) / abs(float(H(t)))
              for t in np.linspace(0, 1, 2001))
    print("// max relative truncation error (double evaluation): %.2e" % err)
    print("{" + ", ".join("%.9ef" % c for c in coef) + "}")


if __name__ == "__main__":
    main()
