"""Generate tests/golden/static_singular.npz: static (k = 0) local matrices of singular triangle
pairs, computed independently of any quadrature code in this repository.

For a test triangle tau and trial triangle sigma the local matrices are

  HH   L_ij = 1/(4 pi) int_tau int_sigma lambda_i(x) lambda_j(y) / |x - y|        (Lagrange hats)
  MWa  L_ij = 1/(4 pi) int_tau int_sigma psi_i(x) . psi_j(y) / |x - y|            (RWG vector part)
  MWb  L_ij = 1/(4 pi) int_tau int_sigma div psi_i div psi_j / |x - y|           (RWG divergence part)
  DL   L_ij = 1/(4 pi) int_tau int_sigma lambda_i(x) lambda_j(y) (x - y).n_sigma / |x - y|^3
  DLT  L_ij = DL of the swapped pair, transposed (the kernel of the transposed double layer)
  MDL  L_ij = 1/(4 pi) int_tau int_sigma psi_i(x) . (grad_x(1/|x - y|) x psi_j(y))      (RWG, MFIE)

with lambda_i the barycentric coordinate of chart vertex i, psi_i(x) = (x - v_i) / (2 A) and
div psi_i = 1 / A (BEAST's RT reference shapes).  The inner integrals over sigma are the closed
forms of the potential of a flat triangle with constant and linear densities (Wilton et al.,
IEEE TAP 32(3), 1984; Graglia, IEEE TAP 41(10), 1993):

  int_T 1/R        = sum_edges [ P0 ln((R+ + l+)/(R- + l-)) - |d| (atan(P0 l+ / (R0^2 + |d| R+))
                                                                   - atan(P0 l- / (R0^2 + |d| R-))) ]
  int_T (y - rho)/R = 1/2 sum_edges u_hat [ R0^2 ln((R+ + l+)/(R- + l-)) + l+ R+ - l- R- ]

with the double-layer potential from the signed solid angle (Van Oosterom & Strackee 1983) and the
surface gradient theorem, and the outer integral over tau is a tensor Gauss-Legendre rule in collapsed coordinates on the
three centroid subtriangles of tau, graded toward tau's edges and vertices (where the outer
integrand loses smoothness).  Checked against the closed-form self term of a triangle
(Eibert & Hansen, IEEE TAP 43(12), 1995) to 1e-14.

The mesh is an ellipsoid (icosphere of level 1 scaled by 1, 0.8, 0.6); the pairs cover common
face, common edge and common vertex in several local positions, and four far pairs.  Near pairs
come from two jittered coplanar 4 x 4 plates 0.01 apart and, not coplanar, from a plate and a copy
tilted by 60 degrees 0.02 beside it.  The Maxwell double layer (MFIE) is pinned through the
gradient of the flat-triangle potential.  Run from the repository root:

    python tests/golden/make_static_fixtures.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def tri_potentials(V, r):
    """P0 = int_T 1/|r - y| dy and P1 = int_T (y - r)/|r - y| dy, flat triangle V (3x3), points r (N, 3)."""
    v1, v2, v3 = V
    n = np.cross(v2 - v1, v3 - v1)
    n /= np.linalg.norm(n)
    d = (r - v1) @ n
    rho = r - d[:, None] * n[None, :]
    ad = np.abs(d)
    P0 = np.zeros(len(r))
    P1 = np.zeros((len(r), 3))
    for a, b in ((v1, v2), (v2, v3), (v3, v1)):
        lhat = (b - a) / np.linalg.norm(b - a)
        uhat = np.cross(lhat, n)
        lm, lp = (a - rho) @ lhat, (b - rho) @ lhat
        P = (a - rho) @ uhat
        Rm, Rp = np.linalg.norm(r - a, axis=1), np.linalg.norm(r - b, axis=1)
        R02 = P * P + d * d
        with np.errstate(divide="ignore", invalid="ignore"):
            num = np.where(lp >= 0, Rp + lp, R02 / (Rp - lp))  # R + l without cancellation
            den = np.where(lm >= 0, Rm + lm, R02 / (Rm - lm))
            lg = np.log(num / den)
        lg = np.where(R02 <= 0, 0.0, lg)
        at = np.arctan2(P * lp, R02 + ad * Rp) - np.arctan2(P * lm, R02 + ad * Rm)
        P0 += P * lg - ad * at
        P1 += 0.5 * uhat[None, :] * (R02 * lg + lp * Rp - lm * Rm)[:, None]
    P1 += (rho - r) * P0[:, None]
    return P0, P1


def dl_potentials(V, r):
    """W0 = int_T d / |r - y|^3 dy (the signed solid angle, d = (r - y) . n) and
    W1 = int_T (y - rho) / |r - y|^3 dy = -sum_edges u_hat ln((R+ + l+)/(R- + l-)) (surface
    gradient theorem), for the double-layer potential of a flat triangle."""
    v1, v2, v3 = V
    n = np.cross(v2 - v1, v3 - v1)
    n /= np.linalg.norm(n)
    d = (r - v1) @ n
    rho = r - d[:, None] * n[None, :]
    q = V[None, :, :] - r[:, None, :]
    nq = np.linalg.norm(q, axis=2)
    trip = np.einsum("ij,ij->i", q[:, 0], np.cross(q[:, 1], q[:, 2]))
    den = (nq[:, 0] * nq[:, 1] * nq[:, 2] + np.einsum("ij,ij->i", q[:, 0], q[:, 1]) * nq[:, 2] +
           np.einsum("ij,ij->i", q[:, 0], q[:, 2]) * nq[:, 1] + np.einsum("ij,ij->i", q[:, 1], q[:, 2]) * nq[:, 0])
    W0 = -2 * np.arctan2(trip, den)  # Van Oosterom & Strackee, IEEE TBME 30(2), 1983
    W1 = np.zeros((len(r), 3))
    for a, b in ((v1, v2), (v2, v3), (v3, v1)):
        lhat = (b - a) / np.linalg.norm(b - a)
        uhat = np.cross(lhat, n)
        lm, lp = (a - rho) @ lhat, (b - rho) @ lhat
        P = (a - rho) @ uhat
        Rm, Rp = np.linalg.norm(r - a, axis=1), np.linalg.norm(r - b, axis=1)
        R02 = P * P + d * d
        with np.errstate(divide="ignore", invalid="ignore"):
            num = np.where(lp >= 0, Rp + lp, R02 / (Rp - lp))
            den2 = np.where(lm >= 0, Rm + lm, R02 / (Rm - lm))
            lg = np.log(num / den2)
        lg = np.where(R02 <= 0, 0.0, lg)
        W1 -= uhat[None, :] * lg[:, None]
    return W0, W1, d


def local_static_dl(Vt, Vs, n=40, p=3):
    """DL_ij = 1/(4 pi) int_tau lambda_i(x) int_sigma lambda_j(y) (x - y) . n_sigma / |x - y|^3."""
    return local_static_dl_at(Vt, Vs, *graded_rule(Vt, n, p))


def local_static_dl_at(Vt, Vs, x, w):
    """local_static_dl with the outer integral taken as the sum over the points x (N, 3) with weights w."""
    W0, W1, d = dl_potentials(Vs, x)
    lam_t = barycentric(Vt, x)
    lam_s = barycentric(Vs, x)
    gs = grad_barycentric(Vs)
    dl = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            inner = lam_s[:, j] * W0 + d * (W1 @ gs[j])
            dl[i, j] = np.sum(w * lam_t[:, i] * inner) / (4 * np.pi)
    return dl


def local_static_mfie(Vt, Vs, n=40, p=3):
    """MFIE_ij = 1/(4 pi) int_tau psi_i(x) . (int_sigma grad_x(1/|x - y|) x psi_j(y) dy) with the RWG
    shapes psi = (x - v) / (2 A).  grad_x(1/R) is parallel to x - y, so the inner integral is
    (int_sigma grad_x(1/R)) x (x - w_j) / (2 A_sigma), and int_sigma grad_x(1/R) = W1 - n W0 from the
    double-layer potentials (Graglia 1993)."""
    return local_static_mfie_at(Vt, Vs, *graded_rule(Vt, n, p))


def local_static_mfie_at(Vt, Vs, x, w):
    """local_static_mfie with the outer integral taken as the sum over the points x with weights w."""
    W0, W1, d = dl_potentials(Vs, x)
    v1, v2, v3 = Vs
    nrm = np.cross(v2 - v1, v3 - v1)
    nrm /= np.linalg.norm(nrm)
    grad = W1 - nrm[None, :] * W0[:, None]
    At = 0.5 * np.linalg.norm(np.cross(Vt[1] - Vt[0], Vt[2] - Vt[0]))
    As = 0.5 * np.linalg.norm(np.cross(Vs[1] - Vs[0], Vs[2] - Vs[0]))
    out = np.zeros((3, 3))
    for i in range(3):
        psi_i = (x - Vt[i]) / (2 * At)
        for j in range(3):
            inner = np.cross(grad, (x - Vs[j]) / (2 * As))
            out[i, j] = np.sum(w * np.einsum("kc,kc->k", psi_i, inner)) / (4 * np.pi)
    return out


def graded_rule(V, n=40, p=3):
    g, gw = np.polynomial.legendre.leggauss(n)
    g, gw = (g + 1) / 2, gw / 2
    s, ds = 1 - (1 - g) ** p, p * (1 - g) ** (p - 1)
    t = g ** p / (g ** p + (1 - g) ** p)
    dt = p * (g * (1 - g)) ** (p - 1) / (g ** p + (1 - g) ** p) ** 2
    c = V.mean(axis=0)
    pts, wts = [], []
    for a, b in ((V[0], V[1]), (V[1], V[2]), (V[2], V[0])):
        asub = 0.5 * np.linalg.norm(np.cross(a - c, b - c))
        S, T = np.meshgrid(s, t, indexing="ij")
        W = np.outer(gw * ds, gw * dt)
        X = c + S[..., None] * ((a - c) + T[..., None] * (b - a))
        pts.append(X.reshape(-1, 3))
        wts.append((W * 2 * asub * S).reshape(-1))
    return np.concatenate(pts), np.concatenate(wts)


def closed_form_self(V):
    a, b, c = (np.linalg.norm(V[1] - V[2]), np.linalg.norm(V[2] - V[0]), np.linalg.norm(V[0] - V[1]))
    A = 0.5 * np.linalg.norm(np.cross(V[1] - V[0], V[2] - V[0]))
    f = lambda a, b, c: np.log(((a + b) ** 2 - c ** 2) / (b ** 2 - (c - a) ** 2)) / a
    return 4 * A * A / 3 * (f(a, b, c) + f(b, c, a) + f(c, a, b))


def barycentric(V, x):
    """Barycentric coordinates of the projections of x (N, 3) on the plane of V."""
    e1, e2 = V[0] - V[2], V[1] - V[2]
    G = np.array([[e1 @ e1, e1 @ e2], [e1 @ e2, e2 @ e2]])
    rhs = np.stack([(x - V[2]) @ e1, (x - V[2]) @ e2], axis=1)
    uv = np.linalg.solve(G, rhs.T).T
    return np.stack([uv[:, 0], uv[:, 1], 1 - uv[:, 0] - uv[:, 1]], axis=1)


def grad_barycentric(V):
    A2 = np.cross(V[1] - V[0], V[2] - V[0])
    n = A2 / np.linalg.norm(A2)
    twoA = np.linalg.norm(A2)
    return np.stack([np.cross(n, V[(j + 2) % 3] - V[(j + 1) % 3]) / twoA for j in range(3)])


def local_static(Vt, Vs, n=40, p=3):
    return local_static_at(Vt, Vs, *graded_rule(Vt, n, p))


def local_static_at(Vt, Vs, x, w):
    """(HH, MW alpha part, MW beta part) with the outer integral as the sum over the points x, weights w."""
    P0, P1 = tri_potentials(Vs, x)
    At = 0.5 * np.linalg.norm(np.cross(Vt[1] - Vt[0], Vt[2] - Vt[0]))
    As = 0.5 * np.linalg.norm(np.cross(Vs[1] - Vs[0], Vs[2] - Vs[0]))
    lam_t = barycentric(Vt, x)
    lam_s = barycentric(Vs, x)
    gs = grad_barycentric(Vs)
    inv4pi = 1 / (4 * np.pi)
    hh = np.zeros((3, 3))
    mwa = np.zeros((3, 3))
    for i in range(3):
        psi_i = (x - Vt[i]) / (2 * At)
        for j in range(3):
            inner_l = lam_s[:, j] * P0 + P1 @ gs[j]
            hh[i, j] = inv4pi * np.sum(w * lam_t[:, i] * inner_l)
            inner_v = (P1 + (x - Vs[j]) * P0[:, None]) / (2 * As)
            mwa[i, j] = inv4pi * np.sum(w * np.einsum("kc,kc->k", psi_i, inner_v))
    mwb = np.full((3, 3), inv4pi * np.sum(w * P0) / (At * As))
    return hh, mwa, mwb


def pick_pairs(tris):
    """CF, CE and CV pairs (tau, sigma) with varied local positions of the shared vertices."""
    nt = len(tris)
    sets = [set(t) for t in tris]
    cf = [(t, t) for t in (0, 17, 53)]
    ce, cv = [], []
    for a in range(nt):
        for b in range(nt):
            if a == b:
                continue
            k = len(sets[a] & sets[b])
            if k == 2 and len(ce) < 6 and a in (0, 5, 23, 41, 60, 77):
                ce.append((a, b))
            elif k == 1 and len(cv) < 6 and a in (2, 9, 30, 44, 66, 71):
                cv.append((a, b))
    return cf + ce[:6] + cv[:6]


def tables(V, T, pairs):
    hh, mwa, mwb, dl, dlt, mdl, err = [], [], [], [], [], [], []
    for a, b in pairs:
        A, B = V[T[a]], V[T[b]]
        r40 = local_static(A, B, 40)
        r60 = local_static(A, B, 60)
        hh.append(r60[0]), mwa.append(r60[1]), mwb.append(r60[2])
        err.append(max(np.abs(x - y).max() / np.abs(y).max() for x, y in zip(r40, r60)))
        if a == b:  # the double layers vanish on a flat common face
            dl.append(np.zeros((3, 3))), dlt.append(np.zeros((3, 3))), mdl.append(np.zeros((3, 3)))
            continue
        d40, d60 = local_static_dl(A, B, 40), local_static_dl(A, B, 60)
        t60 = local_static_dl(B, A, 60).T  # transposed double layer: DL with the roles swapped
        # the MFIE's outer integrand has a logarithmic edge singularity on common-edge pairs: more points
        m80, m100 = local_static_mfie(A, B, 80), local_static_mfie(A, B, 100)
        dl.append(d60), dlt.append(t60), mdl.append(m100)
        for x, y in ((d40, d60), (m80, m100)):
            sc = np.abs(y).max()
            if sc > 1e-14 * np.abs(r60[0]).max():  # coplanar pairs: the double layers vanish
                err.append(np.abs(x - y).max() / sc)
    return (np.array(hh), np.array(mwa), np.array(mwb), np.array(dl), np.array(dlt), np.array(mdl), np.array(err))


def tilted_plates(n=4, jitter=0.3, seed=1, gap=0.02, angle=np.pi / 3):
    """A jittered n x n plate in z = 0 and a copy turned by `angle` about the x axis, lifted so that
    its lower edge runs `gap` above and beside the first plate's edge y = 1: near pairs that are
    not coplanar (the double layers do not vanish)."""
    import beastgpu_gb300 as bg
    p = bg.plate(n, jitter, seed)
    v = p.vertices.copy()
    c, s = np.cos(angle), np.sin(angle)
    q = np.stack([v[:, 0], 1.0 + gap + c * v[:, 1], gap + s * v[:, 1]], axis=1)
    return np.concatenate([v, q]), np.concatenate([p.triangles, p.triangles + p.nv]).astype(np.int32)


def main():
    import beastgpu_gb300 as bg
    m = bg.ellipsoid(1, (1.0, 0.8, 0.6))
    V, T = m.vertices.astype(np.float64), m.triangles.astype(np.int32)
    pairs = pick_pairs(T.tolist())
    assert len(pairs) == 15, len(pairs)
    # far pairs: the three closest non-touching pairs and the farthest one
    pairs += [(67, 69), (40, 55), (3, 12), (19, 59)]
    hh, mwa, mwb, dl, dlt, mdl, err = tables(V, T, pairs)
    # near pairs (class 4 at k = 0) of two jittered coplanar 4 x 4 plates 0.01 apart
    p = bg.two_plates(4, jitter=0.3, seed=1, gap=0.01)
    PV, PT = p.vertices.astype(np.float64), p.triangles.astype(np.int32)
    near = [(24, 32), (25, 34), (26, 37), (24, 35)]
    nhh, nmwa, nmwb, ndl, ndlt, nmdl, nerr = tables(PV, PT, near)
    # near pairs across a plate and a tilted copy (not coplanar), at gaps 0.02 .. 0.1 of the plate
    tv, tt = tilted_plates()
    tilted = [(6, 32), (7, 33), (14, 48), (15, 41), (23, 56), (31, 57)]
    thh, tmwa, tmwb, tdl, tdlt, tmdl, terr = tables(tv, tt, tilted)
    # the CF self term of the outer rule against its closed form
    Vt = V[T[0]]
    x, w = graded_rule(Vt, 60)
    P0, _ = tri_potentials(Vt, x)
    self_err = abs(np.sum(w * P0) - closed_form_self(Vt)) / closed_form_self(Vt)
    out = os.path.join(HERE, "static_singular.npz")
    np.savez(out, vertices=V, triangles=T, tau=np.array([q[0] for q in pairs], dtype=np.int32),
             sigma=np.array([q[1] for q in pairs], dtype=np.int32), hh=hh, mw_alpha=mwa, mw_beta=mwb, dl=dl, dlt=dlt,
             mw_dl=mdl, plate_vertices=PV, plate_triangles=PT, near_tau=np.array([q[0] for q in near], dtype=np.int32),
             near_sigma=np.array([q[1] for q in near], dtype=np.int32), near_hh=nhh, near_mw_alpha=nmwa,
             near_mw_beta=nmwb, near_dl=ndl, near_dlt=ndlt, near_mw_dl=nmdl, tilted_vertices=tv, tilted_triangles=tt,
             tilted_tau=np.array([q[0] for q in tilted], dtype=np.int32),
             tilted_sigma=np.array([q[1] for q in tilted], dtype=np.int32), tilted_hh=thh, tilted_mw_alpha=tmwa,
             tilted_mw_beta=tmwb, tilted_dl=tdl, tilted_dlt=tdlt, tilted_mw_dl=tmdl,
             rule_change=np.concatenate([err, nerr, terr]), self_term_error=np.array(self_err))
    print(f"wrote {out}: {len(pairs)} + {len(near)} + {len(tilted)} pairs, max change 40 -> 60 (MFIE 80 -> 100) points per dimension "
          f"{max(err.max(), nerr.max(), terr.max()):.2e}, self-term error {self_err:.2e}")


if __name__ == "__main__":
    main()
