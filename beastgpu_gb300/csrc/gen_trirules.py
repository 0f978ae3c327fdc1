"""Generate the symmetric triangle quadrature tables used by the library and the oracle.

The rules are D. A. Dunavant's symmetric Gaussian rules for the triangle ("High degree
efficient symmetrical Gaussian quadrature rules for the triangle", IJNME 21, 1985) of
degree 1..7 (1, 3, 4, 6, 7, 12, 13 points).  The published decimals are refined here by
Gauss-Newton on the monomial moment equations in 50-digit arithmetic, so every constant
is exact to double precision and each rule integrates all monomials up to its degree.

Points are written as the chart parameters (u, v) of BEAST/CompScienceMeshes, i.e. the
point u*v1 + v*v2 + (1-u-v)*v3 of the triangle (v1, v2, v3); weights sum to one (multiply
by the triangle area to integrate).  Run:  python beastgpu_gb300/csrc/gen_trirules.py
"""
import os
import mpmath as mp

mp.mp.dps = 50
START = {
    1: [("S3", [], 1.0)],
    3: [("S21", [0.166666666666667], 1 / 3.0)],
    4: [("S3", [], -0.5625), ("S21", [0.2], 0.520833333333333)],
    6: [("S21", [0.445948490915965], 0.223381589678011), ("S21", [0.091576213509771], 0.109951743655322)],
    7: [("S3", [], 0.225), ("S21", [0.470142064105115], 0.132394152788506),
        ("S21", [0.101286507323456], 0.125939180544827)],
    12: [("S21", [0.249286745170910], 0.116786275726379), ("S21", [0.063089014491502], 0.050844906370207),
         ("S111", [0.053145049844817, 0.310352451033784], 0.082851075618374)],
    13: [("S3", [], -0.149570044467682), ("S21", [0.260345966079040], 0.175615257433208),
         ("S21", [0.065130102902216], 0.053347235608838),
         ("S111", [0.048690315425316, 0.312865496004874], 0.077113760890257)],
}
DEGREE = {1: 1, 3: 2, 4: 3, 6: 4, 7: 5, 12: 6, 13: 7}


def expand(rule, x):
    pts, k = [], 0
    for (kind, p, _w) in rule:
        ps = x[k:k + len(p)]
        k += len(p)
        w = x[k]
        k += 1
        if kind == "S3":
            pts.append((mp.mpf(1) / 3, mp.mpf(1) / 3, w))
        elif kind == "S21":
            a = ps[0]
            b = 1 - 2 * a
            pts += [(b, a, w), (a, b, w), (a, a, w)]
        else:
            a, b = ps
            c = 1 - a - b
            pts += [(a, b, w), (b, a, w), (a, c, w), (c, a, w), (b, c, w), (c, b, w)]
    return pts


def residual(rule, x, d):
    pts = expand(rule, x)
    r = []
    for i in range(d + 1):
        for j in range(d + 1 - i):
            s = sum(w * u ** i * v ** j for (u, v, w) in pts)
            r.append(s - 2 * mp.factorial(i) * mp.factorial(j) / mp.factorial(i + j + 2))
    return mp.matrix(r)


def refine(n):
    rule = START[n]
    x = []
    for (_k, p, w) in rule:
        x += [mp.mpf(v) for v in p] + [mp.mpf(w)]
    x = mp.matrix(x)
    d = DEGREE[n]
    for _ in range(40):
        r = residual(rule, x, d)
        jac = mp.matrix(len(r), len(x))
        h = mp.mpf(10) ** -30
        for c in range(len(x)):
            xp = x.copy()
            xp[c] += h
            rp = residual(rule, xp, d)
            for q in range(len(r)):
                jac[q, c] = (rp[q] - r[q]) / h
        dx = mp.lu_solve(jac.T * jac, -(jac.T * r))
        x = x + dx
        if mp.norm(dx) < mp.mpf(10) ** -40:
            break
    assert mp.norm(residual(rule, x, d)) < mp.mpf(10) ** -35
    pts = expand(rule, x)
    assert len(pts) == n
    return pts


def emit(guard, prefix):
    lines = [f"/* Generated by beastgpu_gb300/csrc/gen_trirules.py -- do not edit. */",
             "/* Dunavant symmetric triangle rules; (u, v, w): point u*v1 + v*v2 + (1-u-v)*v3, sum w = 1. */",
             f"#ifndef {guard}", f"#define {guard}", "",
             f"#define {prefix.upper()}TRIRULE_COUNT 7",
             f"static const int {prefix}trirule_npoints[7] = {{1, 3, 4, 6, 7, 12, 13}};",
             f"static const int {prefix}trirule_degree[7] = {{1, 2, 3, 4, 5, 6, 7}};",
             f"static const int {prefix}trirule_offset[7] = {{0, 1, 4, 8, 14, 21, 33}};",
             f"static const double {prefix}trirule_uvw[46][3] = {{"]
    for n in (1, 3, 4, 6, 7, 12, 13):
        lines.append(f"  /* {n} points, degree {DEGREE[n]} */")
        for (u, v, w) in refine(n):
            lines.append("  {%s, %s, %s}," % tuple(repr(float(t)) for t in (u, v, w)))
    lines += ["};", "", "#endif", ""]
    return "\n".join(lines)


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(os.path.dirname(here))
    with open(os.path.join(here, "trirules.h"), "w") as f:
        f.write(emit("BGB_TRIRULES_H", "bgb_"))
    with open(os.path.join(root, "oracle", "trirules.h"), "w") as f:
        f.write(emit("ORC_TRIRULES_H", "orc_"))
