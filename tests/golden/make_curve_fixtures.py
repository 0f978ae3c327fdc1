"""Generate tests/golden/curve_pairs.npz: local matrices of segment pairs for the 2-D (curve)
operators, computed by adaptive Gauss-Kronrod quadrature (QUADPACK through scipy.integrate.quad,
nested, with the singular point of the inner integral as a breakpoint) -- independently of the
graded and Gauss-Legendre rules of the oracle and of the library.

For a test segment tau and a trial segment sigma with charts x(s) = a + s d_tau,
y(t) = b + t d_sigma (s, t in [0, 1]), lengths l and normals n = (d_y, -d_x) / l:

  SL_ij  = int int G(R) f_i(s) g_j(t) l_tau l_sigma ds dt
  DL_ij  = int int -((x - y) . n_sigma) g1(R) f_i(s) g_j(t) l_tau l_sigma ds dt
  DLT_ij = int int  ((x - y) . n_tau) g1(R) f_i(s) g_j(t) l_tau l_sigma ds dt

with f = (1 - s, s), g = (1 - t, t), R = |x - y|, G = -(i/4) H0^(2)(kR) and
g1 = (i k / 4) H1^(2)(kR) / R (scipy.special.hankel2), or G = -ln(R) / (2 pi) and
g1 = -1 / (2 pi R^2) for k = 0.  The hypersingular and piecewise-constant matrices are linear
combinations of these (the tests form them).  Double layers vanish on coincident segments.

The pairs (test segment, trial segment) cover coincident segments in the same and in the
opposite orientation, common vertices at several angles and local positions, a near pair
(parallel segments 0.03 apart) and far pairs, for k = 0 and k = 3.  Run from the repository
root:

    python tests/golden/make_curve_fixtures.py
"""
from __future__ import annotations

import os

import numpy as np
from scipy import integrate, special

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "curve_pairs.npz")

VERTICES = np.array([[0.0, 0.0], [0.5, 0.0], [0.9, 0.3], [0.2, 0.45], [0.45, -0.03], [0.95, -0.03],
                     [3.0, 1.0], [3.4, 1.3], [0.5, -0.6], [-0.3, 0.1]])
TEST_SEGMENTS = np.array([[0, 1], [1, 2], [0, 3], [9, 0]])
TRIAL_SEGMENTS = np.array([[0, 1], [1, 0], [1, 2], [3, 0], [2, 1], [8, 1], [4, 5], [6, 7], [1, 8], [0, 9]])
# (tau, sigma, class): 3 coincident, 1 common vertex, 4 near, 0 far
PAIRS = [(0, 0, 3), (0, 1, 3), (1, 2, 3), (1, 4, 3),
         (0, 2, 1), (0, 3, 1), (0, 5, 1), (1, 0, 1), (2, 0, 1), (3, 0, 1), (0, 8, 1), (3, 9, 3), (2, 9, 1),
         (0, 6, 4), (1, 6, 4),
         (0, 7, 0), (2, 7, 0)]
WAVENUMBERS = (0.0, 3.0)


def green(k, R):
    if k == 0.0:
        return -np.log(R) / (2 * np.pi), -1.0 / (2 * np.pi * R * R)
    return -0.25j * special.hankel2(0, k * R), 0.25j * k * special.hankel2(1, k * R) / R


def seg(s):
    a, b = VERTICES[s[0]], VERTICES[s[1]]
    d = b - a
    l = np.linalg.norm(d)
    return a, d, l, np.array([d[1], -d[0]]) / l


def integrate_pair(k, A, B, kind, i, j, part):
    a, dA, lA, nA = A
    b, dB, lB, nB = B
    f = (lambda s: 1 - s, lambda s: s)

    def val(s, t):
        x = a + s * dA
        y = b + t * dB
        r = x - y
        R = np.hypot(r[0], r[1])
        G, g1 = green(k, R)
        K = G if kind == "sl" else (-(r @ nB) * g1 if kind == "dl" else (r @ nA) * g1)
        v = K * f[i](s) * f[j](t) * lA * lB
        return v.real if part == 0 else v.imag

    def inner(s):
        x = a + s * dA
        # breakpoint: the trial parameter of the point of sigma closest to x
        tc = float(np.clip((x - b) @ dB / (dB @ dB), 0.0, 1.0))
        pts = [tc] if 0.0 < tc < 1.0 else None
        return integrate.quad(lambda t: val(s, t), 0.0, 1.0, points=pts, epsabs=1e-15, epsrel=1e-13, limit=400)[0]

    return integrate.quad(inner, 0.0, 1.0, epsabs=1e-15, epsrel=1e-12, limit=400)[0]


def main():
    out = {"vertices": VERTICES, "test_segments": TEST_SEGMENTS, "trial_segments": TRIAL_SEGMENTS,
           "tau": np.array([p[0] for p in PAIRS]), "sigma": np.array([p[1] for p in PAIRS]),
           "cls": np.array([p[2] for p in PAIRS]), "wavenumbers": np.array(WAVENUMBERS)}
    for k in WAVENUMBERS:
        for kind in ("sl", "dl", "dlt"):
            L = np.zeros((len(PAIRS), 2, 2), dtype=np.complex128)
            for p, (t, s, c) in enumerate(PAIRS):
                if kind != "sl" and c == 3:
                    continue
                A, B = seg(TEST_SEGMENTS[t]), seg(TRIAL_SEGMENTS[s])
                for i in range(2):
                    for j in range(2):
                        re = integrate_pair(k, A, B, kind, i, j, 0)
                        im = integrate_pair(k, A, B, kind, i, j, 1) if k > 0 else 0.0
                        L[p, i, j] = re + 1j * im
            out[f"{kind}_k{int(k)}"] = L
            print(kind, k, "done", flush=True)
    # the same machinery against the closed form int int ln|s - t| = -3/2 (constant functions)
    a, d, l, n = seg(TEST_SEGMENTS[0])
    tot = sum(out["sl_k0"][0].ravel())
    out["closed_form_check"] = np.array(abs(tot - (-(l * l) / (2 * np.pi) * (np.log(l) - 1.5))))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, "closed-form check", float(out["closed_form_check"]))


if __name__ == "__main__":
    main()
