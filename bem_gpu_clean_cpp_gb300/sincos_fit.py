"""Coefficients of the FP64 sin/cos polynomials of the near-field quadrature
(csrc/kernels.cu, sincos_near), derived here rather than taken from a library.

On |z| <= pi/4, with u = z^2:
  sin z = z + z^3 P(u),  P of degree NS - 1   (P(u) ~ (sin(sqrt u) - sqrt u) / u^1.5)
  cos z = 1 - u/2 + u^2 Q(u),  Q of degree NC - 1
P and Q are Chebyshev interpolants of the exact functions on u in [0, (pi/4)^2]
(near-minimax), computed with mpmath at 60 digits, converted to the monomial
basis and rounded to double.  Running this file prints the coefficients and
the maximum error of the double-evaluated Horner schemes on a dense grid.
"""
import mpmath as mp

mp.mp.dps = 60
UMAX = (mp.pi / 4) ** 2


def cheb_fit(f, deg):
    """Monomial coefficients (low to high) of the degree-deg Chebyshev
    interpolant of f on [0, UMAX]."""
    n = deg + 1
    nodes = [UMAX / 2 * (1 + mp.cos(mp.pi * (k + mp.mpf(1) / 2) / n)) for k in range(n)]
    # solve the Vandermonde system exactly in high precision
    A = mp.matrix([[u ** j for j in range(n)] for u in nodes])
    b = mp.matrix([f(u) for u in nodes])
    return list(mp.lu_solve(A, b))


def p_sin(u):  # (sin z - z) / z^3 as a function of u = z^2
    z = mp.sqrt(u)
    return (mp.sin(z) - z) / z ** 3 if u != 0 else mp.mpf(-1) / 6


def q_cos(u):  # (cos z - 1 + u/2) / u^2
    z = mp.sqrt(u)
    return (mp.cos(z) - 1 + u / 2) / u ** 2 if u != 0 else mp.mpf(1) / 24


def max_error(ns, nc, npts=4000):
    P = [float(c) for c in cheb_fit(p_sin, ns - 1)]
    Q = [float(c) for c in cheb_fit(q_cos, nc - 1)]
    worst_s = worst_c = mp.mpf(0)
    for i in range(npts + 1):
        z = float(-mp.pi / 4 + mp.pi / 2 * i / npts)
        u = z * z
        ps = P[-1]
        for c in reversed(P[:-1]):
            ps = ps * u + c
        s = z + (ps * u) * z            # double arithmetic, as on the GPU (FMA aside)
        pc = Q[-1]
        for c in reversed(Q[:-1]):
            pc = pc * u + c
        cval = 1.0 - 0.5 * u + pc * u * u
        worst_s = max(worst_s, abs(mp.mpf(s) - mp.sin(z)))
        worst_c = max(worst_c, abs(mp.mpf(cval) - mp.cos(z)))
    return P, Q, worst_s, worst_c


if __name__ == "__main__":
    for ns, nc in [(6, 6), (7, 7)]:
        P, Q, es, ec = max_error(ns, nc)
        print(f"sin: {ns} coefficients, max abs error {float(es):.3e}; cos: {nc} coefficients, {float(ec):.3e}")
        print("  P =", [repr(c) for c in P])
        print("  Q =", [repr(c) for c in Q])
