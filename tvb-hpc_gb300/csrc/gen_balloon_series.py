"""
Coefficients of the polynomial forms used by the balloon step
(tvbg_device.cuh, Balloon::step):

  (1 + V)^p - 1       = sum_{k=1..8} binom(p, k) V^k         p = 1/alpha, 1/alpha - 1
  g(F) = (1+F)(1 - a^(1/(1+F)))/E0 - 1 = sum_{k=1..8} c_k F^k     a = 1 - E0

(alpha = 0.32, E0 = 0.4: the Stephan et al. 2007 constants of
tvb_hpc/bold.py:24-57).  Run `python gen_balloon_series.py` to print the
constants pasted into the kernel header.
"""

import sympy as sp

ALPHA = sp.Rational(32, 100)
E0 = sp.Rational(4, 10)


def binomial_coeffs(p, n=8):
    return [sp.binomial(p, k) for k in range(1, n + 1)]


def oxygen_coeffs(n=8):
    F = sp.Symbol('F')
    a = 1 - E0
    g = (1 + F) * (1 - a ** (1 / (1 + F))) / E0 - 1
    ser = sp.series(g, F, 0, n + 1).removeO()
    return [sp.N(ser.coeff(F, k), 20) for k in range(1, n + 1)]


def main():
    p1 = 1 / ALPHA
    for name, cs in (('kPowA', binomial_coeffs(p1)), ('kPowB', binomial_coeffs(p1 - 1)),
                     ('kOxy', oxygen_coeffs())):
        vals = ', '.join('%.12ef' % float(c) for c in cs)
        print('constexpr float %s[8] = {%s};' % (name, vals))


if __name__ == '__main__':
    main()
