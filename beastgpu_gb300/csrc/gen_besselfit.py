"""Generate besselfit.h: polynomial approximations of the Hankel functions H0^(2), H1^(2) for the
FP32 point-pair arithmetic of the mixed curve kernels.

The forms are those of the classical approximations in Abramowitz & Stegun (9.4.1-9.4.6): with
u = (x/3)^2 on 0 < x < 3

    J0(x) = P0(u)                      Y0(x) = (2/pi) ln(x/2) J0(x) + Q0(u)
    J1(x) = x P1(u)                    x Y1(x) = (2/pi) x ln(x/2) J1(x) + Q1(u)

and with t = 3/x on x >= 3 the modulus / phase form

    H_nu^(2)(x) = J_nu - i Y_nu = x^(-1/2) F_nu(t) exp(-i theta_nu),
    theta_0 = x - pi/4 + G0(t),        theta_1 = x - 3 pi/4 + G1(t).

The coefficients are fitted here (least squares at 4,000 Chebyshev points, double precision)
against scipy.special's Bessel functions, to absolute errors below 5e-9 (P, Q) and relative /
phase errors below 5e-9 (F, G) at the lowest such degrees: evaluated in FP32 the approximations are
then limited by the single-precision rounding (~1e-7).  Run from the repository root:

    python beastgpu_gb300/csrc/gen_besselfit.py
"""
from __future__ import annotations

import os

import numpy as np
from scipy import special

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "besselfit.h")
X0 = 3.0


def cheb01(n, lo=0.0):
    k = np.arange(n)
    return lo + (1 - lo) * 0.5 * (1 - np.cos(np.pi * (k + 0.5) / n))


def fit(u, y, deg):
    c = np.polynomial.polynomial.polyfit(u, y, deg)
    err = np.abs(np.polynomial.polynomial.polyval(u, c) - y).max()
    return c, err


def small_targets(u):
    x = X0 * np.sqrt(u)
    j0, y0, j1, y1 = special.j0(x), special.y0(x), special.j1(x), special.y1(x)
    with np.errstate(divide="ignore", invalid="ignore"):
        lg = np.log(x / 2)
        q0 = y0 - (2 / np.pi) * lg * j0
        p1 = j1 / x
        q1 = x * y1 - (2 / np.pi) * x * lg * j1
    return j0, q0, p1, q1


def large_targets(t):
    x = X0 / t
    h0 = special.hankel2(0, x)
    h1 = special.hankel2(1, x)
    f0 = np.sqrt(x) * np.abs(h0)
    f1 = np.sqrt(x) * np.abs(h1)
    # H = |H| exp(-i theta): theta - (x - pi/4) = -arg(H exp(i (x - pi/4))), small, no wrap
    g0 = -np.angle(h0 * np.exp(1j * (x - np.pi / 4)))
    g1 = -np.angle(h1 * np.exp(1j * (x - 3 * np.pi / 4)))
    return f0, g0, f1, g1


def main():
    u = cheb01(4000)
    j0, q0, p1, q1 = small_targets(u)
    t = cheb01(4000, lo=1e-5)
    f0, g0, f1, g1 = large_targets(t)
    fits = {}
    # the lowest degrees with errors below 5e-9 (single-precision rounding is ~6e-8)
    for name, uu, y, deg in (("P0", u, j0, 7), ("Q0", u, q0, 7), ("P1", u, p1, 6), ("Q1", u, q1, 7),
                             ("F0", t, f0, 7), ("G0", t, g0, 7), ("F1", t, f1, 7), ("G1", t, g1, 7)):
        c, err = fit(uu, y, deg)
        fits[name] = (c, err)
        print(f"{name}: degree {deg}, max error {err:.2e}")
        assert err < 5e-9, name
    lines = ["// Generated by gen_besselfit.py: polynomial approximations of H0^(2), H1^(2) for FP32",
             "// evaluation (forms of Abramowitz & Stegun 9.4.1-9.4.6, coefficients fitted against",
             "// scipy.special).  Coefficients in ascending powers; x < 3: u = (x/3)^2, x >= 3: t = 3/x.",
             "#pragma once", ""]
    for name, (c, err) in fits.items():
        body = ", ".join(f"{v:.9e}f" for v in c)
        lines.append(f"// max fit error {err:.1e}")
        lines.append(f"#define BGB_BESSEL_{name} {{{body}}}")
        lines.append(f"#define BGB_BESSEL_{name}_N {len(c)}")
    open(OUT, "w").write("\n".join(lines) + "\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
